/* div E correction on the periodic uniform mesh -- FP64 restatement of
 * PIC::FieldSolver::Electromagnetic::ECSIM::divECorrection
 * (src/pic/pic_field_solver_ecsim.cpp:4341-4364).  TEST INFRASTRUCTURE: only
 * tests/ load this library; the product never does.
 *
 * Parity unpinned: the reference exits when DoDivECorrection is set
 * (:6168-6170, its Poisson stencil predates the current linear-system
 * interface), so no reference output exists.  The restatement follows the
 * reference's steps one by one:
 *   ComputeNetCharge :4690-4828 -- each particle's q w (weight correction
 *     included) spread over the 8 cell centres of CellCentered::Linear's
 *     trilinear stencil (pic_interpolation_routines.cpp:820-905: i0 = -1 for
 *     iLoc < 0.5, else (int)(iLoc - 0.5), weight iLoc - (i0 + 0.5)), summed
 *     across block faces, divided by the cell volume; UpdateOldNetCharge keeps
 *     the previous density;
 *   ComputeDivE :1474-1545 -- div E of the corner E at each cell centre, the
 *     four edge differences per axis averaged;
 *   the Poisson system PoissonGetStencil :645-735 (7-point Laplacian on the
 *     cell centres; a periodic domain has no boundary rows) with
 *     PoissonUpdateRhs :6023-6036, rhs = (-4 pi (g rho_new + (1 - g) rho_old)
 *     + div E) / g, g = 0.51, initial guess 0 (PoissonSetInitialGuess :6304);
 *     solved here by conjugate gradients on -Laplacian (the reference's GMRES
 *     wrapper is absent) with the rhs's mean removed (the periodic Laplacian's
 *     null space);
 *   CorrectParticleLocation :4440-4683 -- species 0 only: the corner nearest
 *     the particle, grad phi there from face differences of phi interpolated
 *     bilinearly (interp2D :216-232), the species-0 charge density at that
 *     corner (the reference reads its corner species moments; here they are
 *     summed from the particles being corrected), displacement
 *     -0.9 grad phi / (4 pi rho_e) (0 where rho_e = 0), capped at 0.1 dx, then
 *     re-binning; ComputeNetCharge again (rho_old kept). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "amps_oracle.h"

#define PI_D 3.14159265358979323846
#define GAMMA_DIVE 0.51
#define EPS_DIVE 0.9
#define LIMIT_DIVE 0.1

/* cell / corner index of global lattice indices (periodic wrap): the global
 * order I + NX (J + NY K) of the oracle's corner and cell arrays */
static long gid(const orc_mesh* g, long I, long J, long K) {
  const long NX = 8L * g->nbx, NY = 8L * g->nby, NZ = 8L * g->nbz;
  I = ((I % NX) + NX) % NX;
  J = ((J % NY) + NY) % NY;
  K = ((K % NZ) + NZ) % NZ;
  return I + NX * (J + NY * K);
}

static void block_coords(const orc_mesh* g, int b, long bc[3]) {
  bc[0] = b % g->nbx;
  bc[1] = (b / g->nbx) % g->nby;
  bc[2] = b / (g->nbx * g->nby);
}

/* block-local offset of x in cell units */
static void local_offset(const orc_mesh* g, const long bc[3], const double* x, double u[3]) {
  for (int d = 0; d < 3; d++) u[d] = (x[d] - (g->x0[d] + 8.0 * bc[d] * g->dx[d])) / g->dx[d];
}

void orc_net_charge(const orc_mesh* g, long n, const double* x, const uint8_t* spec,
                    const double* wcorr, const int32_t* block, double* rho) {
  const long nc = 512L * g->nbx * g->nby * g->nbz;
  memset(rho, 0, sizeof(double) * (size_t)nc);
  const double V = g->dx[0] * g->dx[1] * g->dx[2];
  for (long p = 0; p < n; p++) {
    if (block[p] < 0) continue;
    long bc[3];
    block_coords(g, block[p], bc);
    double u[3];
    local_offset(g, bc, x + 3 * p, u);
    long i0[3];
    double w[3];
    for (int d = 0; d < 3; d++) {
      i0[d] = u[d] < 0.5 ? -1 : (long)(u[d] - 0.5);
      w[d] = u[d] - ((double)i0[d] + 0.5);
    }
    const int s = spec[p];
    const double q = g->q[s] * g->w[s] * (wcorr ? wcorr[p] : 1.0);
    for (int c = 0; c < 2; c++)
      for (int b = 0; b < 2; b++)
        for (int a = 0; a < 2; a++) {
          const double W = (a ? w[0] : 1.0 - w[0]) * (b ? w[1] : 1.0 - w[1]) * (c ? w[2] : 1.0 - w[2]);
          rho[gid(g, 8 * bc[0] + i0[0] + a, 8 * bc[1] + i0[1] + b, 8 * bc[2] + i0[2] + c)] += W * q;
        }
  }
  for (long c = 0; c < nc; c++) rho[c] /= V;
}

/* corner order of ComputeDivE: (i,j,k) (i+1,j,k) (i+1,j+1,k) (i,j+1,k), then k+1 */
static const int kCo[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                              {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

void orc_div_e(const orc_mesh* g, const double* E, double* dive) {
  const int pos[3][4] = {{1, 2, 5, 6}, {2, 3, 6, 7}, {4, 5, 6, 7}};
  const int neg[3][4] = {{0, 3, 4, 7}, {0, 1, 4, 5}, {0, 1, 2, 3}};
  for (int b = 0; b < g->nbx * g->nby * g->nbz; b++) {
    long bc[3];
    block_coords(g, b, bc);
    for (int l = 0; l < 512; l++) {
      const long I = 8 * bc[0] + (l & 7), J = 8 * bc[1] + ((l >> 3) & 7), K = 8 * bc[2] + (l >> 6);
      long co[8];
      for (int c = 0; c < 8; c++) co[c] = gid(g, I + kCo[c][0], J + kCo[c][1], K + kCo[c][2]);
      double s = 0.0;
      for (int d = 0; d < 3; d++)
        for (int t = 0; t < 4; t++) s += (E[3 * co[pos[d][t]] + d] - E[3 * co[neg[d][t]] + d]) / g->dx[d];
      dive[gid(g, I, J, K)] = 0.25 * s;
    }
  }
}

void orc_poisson_rhs(const orc_mesh* g, const double* rho_new, const double* rho_old,
                     const double* dive, double* rhs) {
  const long nc = 512L * g->nbx * g->nby * g->nbz;
  for (long c = 0; c < nc; c++)
    rhs[c] = (-4.0 * PI_D * (GAMMA_DIVE * rho_new[c] + (1.0 - GAMMA_DIVE) * rho_old[c]) + dive[c]) /
             GAMMA_DIVE;
}

/* y = -Laplacian(x), 7 points */
static void neg_lap(const orc_mesh* g, const double* x, double* y) {
  const double c2[3] = {1.0 / (g->dx[0] * g->dx[0]), 1.0 / (g->dx[1] * g->dx[1]),
                        1.0 / (g->dx[2] * g->dx[2])};
  for (int b = 0; b < g->nbx * g->nby * g->nbz; b++) {
    long bc[3];
    block_coords(g, b, bc);
    for (int l = 0; l < 512; l++) {
      const long I = 8 * bc[0] + (l & 7), J = 8 * bc[1] + ((l >> 3) & 7), K = 8 * bc[2] + (l >> 6);
      const long c = gid(g, I, J, K);
      double s = 2.0 * (c2[0] + c2[1] + c2[2]) * x[c];
      s -= c2[0] * (x[gid(g, I - 1, J, K)] + x[gid(g, I + 1, J, K)]);
      s -= c2[1] * (x[gid(g, I, J - 1, K)] + x[gid(g, I, J + 1, K)]);
      s -= c2[2] * (x[gid(g, I, J, K - 1)] + x[gid(g, I, J, K + 1)]);
      y[c] = s;
    }
  }
}

static double dot(long n, const double* a, const double* b) {
  double s = 0.0;
  for (long i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* Laplacian(phi) = rhs: CG on -Laplacian(phi) = -rhs + mean(rhs), phi0 = 0,
 * until ||r|| <= tol ||f||.  Returns the iterations; *rel the final ||r||/||f||. */
int orc_poisson_cg(const orc_mesh* g, const double* rhs, double* phi, double tol, int maxit,
                   double* rel) {
  const long nc = 512L * g->nbx * g->nby * g->nbz;
  double* f = (double*)malloc(sizeof(double) * (size_t)nc * 4);
  double *r = f + nc, *pv = f + 2 * nc, *Ap = f + 3 * nc;
  double mean = 0.0;
  for (long c = 0; c < nc; c++) mean += rhs[c];
  mean /= (double)nc;
  for (long c = 0; c < nc; c++) {
    f[c] = -(rhs[c] - mean);
    phi[c] = 0.0;
    r[c] = f[c];
    pv[c] = f[c];
  }
  const double fn = sqrt(dot(nc, f, f));
  double rr = dot(nc, r, r);
  int it = 0;
  while (it < maxit && sqrt(rr) > tol * fn) {
    neg_lap(g, pv, Ap);
    const double alpha = rr / dot(nc, pv, Ap);
    for (long c = 0; c < nc; c++) {
      phi[c] += alpha * pv[c];
      r[c] -= alpha * Ap[c];
    }
    const double rr1 = dot(nc, r, r);
    const double beta = rr1 / rr;
    for (long c = 0; c < nc; c++) pv[c] = r[c] + beta * pv[c];
    rr = rr1;
    it++;
  }
  if (rel) *rel = fn > 0.0 ? sqrt(rr) / fn : 0.0;
  free(f);
  return it;
}

/* charge density of species s0 at the corners (the 8 corner weights of each
 * particle's cell, q w wc / V) */
void orc_corner_charge(const orc_mesh* g, long n, const double* x, const uint8_t* spec,
                       const double* wcorr, const int32_t* block, const int32_t* cell, int s0,
                       double* cq) {
  const long nc = 512L * g->nbx * g->nby * g->nbz;
  memset(cq, 0, sizeof(double) * (size_t)nc);
  const double V = g->dx[0] * g->dx[1] * g->dx[2];
  for (long p = 0; p < n; p++) {
    if (block[p] < 0 || spec[p] != s0) continue;
    long bc[3];
    block_coords(g, block[p], bc);
    const int i = cell[p] & 7, j = (cell[p] >> 3) & 7, k = cell[p] >> 6;
    double u[3];
    local_offset(g, bc, x + 3 * p, u);
    const double f[3] = {u[0] - i, u[1] - j, u[2] - k};
    const double q = g->q[s0] * g->w[s0] * (wcorr ? wcorr[p] : 1.0) / V;
    for (int c = 0; c < 8; c++) {
      const double W = (kCo[c][0] ? f[0] : 1.0 - f[0]) * (kCo[c][1] ? f[1] : 1.0 - f[1]) *
                       (kCo[c][2] ? f[2] : 1.0 - f[2]);
      cq[gid(g, 8 * bc[0] + i + kCo[c][0], 8 * bc[1] + j + kCo[c][1], 8 * bc[2] + k + kCo[c][2])] += W * q;
    }
  }
}

static double interp2d(double vmm, double vpm, double vpp, double vmp, double a, double b) {
  return vmm * (1 - a) * (1 - b) + vpm * a * (1 - b) + vpp * a * b + vmp * (1 - a) * b;
}

/* CorrectParticleLocation's displacement of the species-0 particles; positions
 * wrapped into the periodic box (block/cell are re-located by the caller).
 * Returns the number of particles displaced. */
long orc_dive_correct(const orc_mesh* g, long n, double* x, const uint8_t* spec,
                      const int32_t* block, const int32_t* cell, const double* phi,
                      const double* cq) {
  long moved = 0;
  const double L[3] = {8.0 * g->nbx * g->dx[0], 8.0 * g->nby * g->dx[1], 8.0 * g->nbz * g->dx[2]};
  for (long p = 0; p < n; p++) {
    if (block[p] < 0 || spec[p] != 0) continue;
    long bc[3];
    block_coords(g, block[p], bc);
    const long idx[3] = {cell[p] & 7, (cell[p] >> 3) & 7, cell[p] >> 6};
    double u[3];
    local_offset(g, bc, x + 3 * p, u);
    double xr[3];
    long ic[3];
    for (int d = 0; d < 3; d++) {
      xr[d] = u[d] - (double)idx[d];
      ic[d] = idx[d] + (long)round(xr[d]);
      xr[d] = xr[d] >= 0.5 ? xr[d] - 0.5 : xr[d] + 0.5;
    }
    /* Phi[ix][iy][iz] with ix = ic + 1 is the centre ic; Phi[ix - 1] the centre ic - 1 */
    const long I = 8 * bc[0] + ic[0], J = 8 * bc[1] + ic[1], K = 8 * bc[2] + ic[2];
#define PH(a, b, c) phi[gid(g, I - 1 + (a), J - 1 + (b), K - 1 + (c))]
    double gp[3];
    gp[0] = interp2d(PH(1, 0, 0) - PH(0, 0, 0), PH(1, 1, 0) - PH(0, 1, 0), PH(1, 1, 1) - PH(0, 1, 1),
                     PH(1, 0, 1) - PH(0, 0, 1), xr[1], xr[2]);
    gp[1] = interp2d(PH(0, 1, 0) - PH(0, 0, 0), PH(1, 1, 0) - PH(1, 0, 0), PH(1, 1, 1) - PH(1, 0, 1),
                     PH(0, 1, 1) - PH(0, 0, 1), xr[0], xr[2]);
    gp[2] = interp2d(PH(0, 0, 1) - PH(0, 0, 0), PH(1, 0, 1) - PH(1, 0, 0), PH(1, 1, 1) - PH(1, 1, 0),
                     PH(0, 1, 1) - PH(0, 1, 0), xr[0], xr[1]);
#undef PH
    for (int d = 0; d < 3; d++) gp[d] /= g->dx[d];
    const double rho_e = cq[gid(g, I, J, K)];
    const double t = rho_e != 0.0 ? 1.0 / (4.0 * PI_D * rho_e) : 0.0;
    double disp[3];
    for (int d = 0; d < 3; d++) disp[d] = -EPS_DIVE * gp[d] * t;
    if (fabs(disp[0] / g->dx[0]) > LIMIT_DIVE || fabs(disp[1] / g->dx[1]) > LIMIT_DIVE ||
        fabs(disp[2] / g->dx[2]) > LIMIT_DIVE) {
      const double dl = sqrt(disp[0] * disp[0] + disp[1] * disp[1] + disp[2] * disp[2]);
      for (int d = 0; d < 3; d++) disp[d] *= LIMIT_DIVE * g->dx[0] / dl;
    }
    for (int d = 0; d < 3; d++) {
      double xn = x[3 * p + d] + disp[d];
      const double rel = xn - g->x0[d];
      if (rel < 0.0) xn += L[d];
      else if (rel >= L[d]) xn -= L[d];
      x[3 * p + d] = xn;
    }
    moved++;
  }
  return moved;
}

/* The whole correction.  rho_new / rho_old persist between calls (first != 0:
 * rho_new is computed first, as the reference's first cycle does).  stats:
 * [0] CG iterations, [1] CG relative residual, [2] ||div E - 4 pi rho_blend||
 * before, [3] after (rho_blend = g rho_new + (1 - g) rho_old), [4] particles
 * displaced. */
void orc_div_e_correction(const orc_mesh* g, long n, double* x, const uint8_t* spec,
                          const double* wcorr, int32_t* block, int32_t* cell, const double* E,
                          double* rho_new, double* rho_old, double* dive, double* phi, int first,
                          double tol, int maxit, double* stats) {
  const long nc = 512L * g->nbx * g->nby * g->nbz;
  double* rhs = (double*)malloc(sizeof(double) * (size_t)nc * 2);
  double* cq = rhs + nc;
  if (first) orc_net_charge(g, n, x, spec, wcorr, block, rho_new);
  memcpy(rho_old, rho_new, sizeof(double) * (size_t)nc);
  orc_net_charge(g, n, x, spec, wcorr, block, rho_new);
  orc_div_e(g, E, dive);
  double before = 0.0, after = 0.0;
  for (long c = 0; c < nc; c++) {
    const double r = dive[c] - 4.0 * PI_D * (GAMMA_DIVE * rho_new[c] + (1.0 - GAMMA_DIVE) * rho_old[c]);
    before += r * r;
  }
  orc_poisson_rhs(g, rho_new, rho_old, dive, rhs);
  double rel = 0.0;
  const int it = orc_poisson_cg(g, rhs, phi, tol, maxit, &rel);
  orc_corner_charge(g, n, x, spec, wcorr, block, cell, 0, cq);
  const long moved = orc_dive_correct(g, n, x, spec, block, cell, phi, cq);
  orc_locate(g, n, x, block, cell);
  orc_net_charge(g, n, x, spec, wcorr, block, rho_new);
  for (long c = 0; c < nc; c++) {
    const double r = dive[c] - 4.0 * PI_D * (GAMMA_DIVE * rho_new[c] + (1.0 - GAMMA_DIVE) * rho_old[c]);
    after += r * r;
  }
  stats[0] = it;
  stats[1] = rel;
  stats[2] = sqrt(before);
  stats[3] = sqrt(after);
  stats[4] = (double)moved;
  free(rhs);
}
