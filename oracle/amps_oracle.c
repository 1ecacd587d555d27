/*
 * amps_oracle.c -- FP64 CPU restatement of the AMPS particle / ECSIM hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see amps_oracle.h).  Deterministic, single
 * threaded, plain C99.  Built with -ffp-contract=off so x86 and Arm hosts
 * give identical results.
 *
 * Index conventions
 *   corner / cell arrays are global and periodic: idx(I,J,K) = I + NX*(J + NY*K),
 *   NX = 8*nbx.  Cell (I,J,K) has its low corner at corner (I,J,K).
 *   Particle cell ids are block-local: i + 8*(j + 8*k); block ids are
 *   bx + nbx*(by + nby*bz).
 *   Per-corner mass matrix: 27 neighbour slots x 9 (row-major 3x3), neighbour
 *   slot n = ii + 3*jj + 9*kk where ii,jj,kk in {0,1,2} stand for offsets
 *   {0,-1,+1} (pic_field_solver_ecsim.cpp:624-640, computeMassMatrixOffsetTable).
 */
#include "amps_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NC ORC_NC
#define PI_D 3.14159265358979323846264338327950288

static int wrap(int i, int n) { i %= n; return i < 0 ? i + n : i; }

/* Open axes (bit d): a particle whose move leaves the domain through a face
 * of such an axis is deleted (the mover's DELETE processing when findTreeNode
 * finds no block, pic_mover_boris.cpp:1159-1170, 1251-1254); block and cell
 * become -1 and every later stage skips it.  Other axes are periodic. */
int orc_open_axes = 0;
void orc_set_open_axes(int mask) { orc_open_axes = mask; }

static long cidx(const orc_mesh* g, int I, int J, int K) {
  const int NX = NC * g->nbx, NY = NC * g->nby, NZ = NC * g->nbz;
  return (long)wrap(I, NX) + (long)NX * ((long)wrap(J, NY) + (long)NY * wrap(K, NZ));
}

/* offset {-1,0,+1} -> slot digit {1,0,2} (reversed_indexAddition, get_stencil.cpp) */
static int slot_digit(int off) { return off == 0 ? 0 : (off < 0 ? 1 : 2); }
static int slot_of(int di, int dj, int dk) {
  return slot_digit(di) + 3 * slot_digit(dj) + 9 * slot_digit(dk);
}

/* corner order of the per-cell tables (InterpolationCoefficientTable order,
 * pic_interpolation_routines.cpp:1112-1145 and ProcessCell offset[] :2033-2040) */
static const int kCornerOff[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                     {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

/* ------------------------------------------------------------------------
 * Stencil tables.  InitDiscritizationStencil (pic_field_solver_ecsim.cpp:7121)
 * builds d2E/dx2 as a second difference along x smoothed by (1/4,1/2,1/4)
 * along the two other axes, and d2E/dxdy as central first differences along
 * x and y smoothed by (1/4,1/2,1/4) along z.  Here the same tables are formed
 * directly as separable products.
 * ---------------------------------------------------------------------- */
static double tap_s(int o) { return o == 0 ? 0.5 : 0.25; }
static double tap_d2(int o) { return o == 0 ? -2.0 : 1.0; }
static double tap_d1(int o) { return o == 0 ? 0.0 : (o > 0 ? 0.5 : -0.5); }

void orc_laplacian_table(int axis, double out[27]) {
  for (int dk = -1; dk <= 1; dk++)
    for (int dj = -1; dj <= 1; dj++)
      for (int di = -1; di <= 1; di++) {
        int o[3] = {di, dj, dk};
        double a = 1.0;
        for (int d = 0; d < 3; d++) a *= (d == axis) ? tap_d2(o[d]) : tap_s(o[d]);
        out[slot_of(di, dj, dk)] = a;
      }
}

void orc_graddiv_table(int p, int q, double out[27]) {
  if (p == q) { orc_laplacian_table(p, out); return; }
  for (int dk = -1; dk <= 1; dk++)
    for (int dj = -1; dj <= 1; dj++)
      for (int di = -1; di <= 1; di++) {
        int o[3] = {di, dj, dk};
        double a = 1.0;
        for (int d = 0; d < 3; d++) a *= (d == p || d == q) ? tap_d1(o[d]) : tap_s(o[d]);
        out[slot_of(di, dj, dk)] = a;
      }
}

/* Operator taps without the mass matrix (GetStencil, get_stencil.cpp:955-1044):
 * K[p][q][slot] = delta_pq*delta_slot0 - delta_pq*sum_d cs[d]*Lap_d + c[p]c[q]*GD_pq */
static void operator_taps(const orc_mesh* g, double K[3][3][27], int with_identity) {
  double coeff[3], cs[3], lap[3][27], gd[27];
  for (int d = 0; d < 3; d++) {
    coeff[d] = g->dt / g->dx[d] * g->theta; /* cDt/dx*theta, c = 1 */
    cs[d] = coeff[d] * coeff[d];
    orc_laplacian_table(d, lap[d]);
  }
  for (int p = 0; p < 3; p++)
    for (int q = 0; q < 3; q++) {
      orc_graddiv_table(p, q, gd);
      for (int s = 0; s < 27; s++) {
        double a = 0.0;
        if (p == q) {
          for (int d = 0; d < 3; d++) a -= lap[d][s] * cs[d];
          if (s == 0 && with_identity) a += 1.0;
        }
        a += gd[s] * coeff[p] * coeff[q];
        K[p][q][s] = a;
      }
    }
}

/* ------------------------------------------------------------------------
 * Corner-based stencil (CornerBased::InitStencil, pic_interpolation_routines.cpp:1074-1194).
 * x is clamped in place exactly like the reference (the caller's copy).
 * Returns the raw trilinear weights in table order, the normalised weights in
 * AddCell order (i outer, k inner), and the base corner index.
 * ---------------------------------------------------------------------- */
static int corner_stencil(const double xmin[3], const double dxc[3], double x[3],
                          double wtab[8], double wnorm[8], int nd[8][3], int iX[3]) {
  double xLoc[3];
  int bad = 0;
  for (int d = 0; d < 3; d++) {
    double xmax = xmin[d] + NC * dxc[d];
    if (x[d] < xmin[d] || x[d] > xmax) bad = 1;
    if (fabs(x[d] - xmax) < 1e-10 * dxc[d]) x[d] = xmax - 1e-10 * dxc[d];
    xLoc[d] = (x[d] - xmin[d]) / dxc[d];
    iX[d] = (int)xLoc[d];
    xLoc[d] -= iX[d];
  }
  int len = 0;
  double norm = 0.0;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++)
      for (int c = 0; c < 2; c++) {
        double w = (a ? xLoc[0] : 1.0 - xLoc[0]);
        w *= (b ? xLoc[1] : 1.0 - xLoc[1]);
        w *= (c ? xLoc[2] : 1.0 - xLoc[2]);
        /* reference evaluates e.g. xLoc[0]*(1-xLoc[1])*(1-xLoc[2]) left to right */
        int t;
        switch (a + 2 * b + 4 * c) {
          case 0: t = 0; break;
          case 1: t = 1; break;
          case 2: t = 3; break;
          case 3: t = 2; break;
          case 4: t = 4; break;
          case 5: t = 5; break;
          case 6: t = 7; break;
          default: t = 6; break;
        }
        wtab[t] = w;
        wnorm[len] = w;
        nd[len][0] = a; nd[len][1] = b; nd[len][2] = c;
        len++;
      }
  for (int s = 0; s < 8; s++) norm += wnorm[s];
  if (norm > 0.0)
    for (int s = 0; s < 8; s++) wnorm[s] /= norm;
  return bad;
}

void orc_corner_weights(const double xloc[3], double w_table[8]) {
  double xmin[3] = {0, 0, 0}, dxc[3] = {1, 1, 1}, x[3], wn[8];
  int nd[8][3], iX[3];
  for (int d = 0; d < 3; d++) x[d] = xloc[d];
  corner_stencil(xmin, dxc, x, w_table, wn, nd, iX);
}

static void block_geom(const orc_mesh* g, int b, int bxyz[3], double xmin[3]) {
  bxyz[0] = b % g->nbx;
  bxyz[1] = (b / g->nbx) % g->nby;
  bxyz[2] = b / (g->nbx * g->nby);
  for (int d = 0; d < 3; d++) xmin[d] = g->x0[d] + bxyz[d] * (NC * g->dx[d]);
}

/* Block containment (findTreeNode, meshAMRgeneric.h:2852-2883: half-open
 * [xmin,xmax) after the +-1 fix-up) and FindCellIndex (:2256-2320). Periodic
 * boundaries follow Periodic::ExchangeParticlesLocal (pic_bc_periodic.cpp:86-178):
 * the cell index is taken in the ghost block, then x is shifted by the
 * block displacement and clamped into the real block. */
static void locate_one(const orc_mesh* g, double x[3], int32_t* blk, int32_t* cel) {
  const int nb[3] = {g->nbx, g->nby, g->nbz};
  int bx[3], ic[3];
  for (int d = 0; d < 3; d++) {
    double L = NC * g->dx[d];
    int b = (int)floor((x[d] - g->x0[d]) / L);
    double xmin = g->x0[d] + b * L;
    if (x[d] < xmin) { b--; xmin = g->x0[d] + b * L; }
    if (x[d] >= xmin + L) { b++; xmin = g->x0[d] + b * L; }
    int i = (int)((x[d] - xmin) / g->dx[d]);
    if (i == NC) i = NC - 1;
    if (b < 0 || b >= nb[d]) {
      int br = wrap(b, nb[d]);
      double xr = g->x0[d] + br * L;
      x[d] += xr - xmin;
      if (x[d] < xr) x[d] = xr;
      if (x[d] >= xr + L) x[d] = (xr + L) - 1.0E-10 * L;
      b = br;
    }
    bx[d] = b;
    ic[d] = i;
  }
  *blk = bx[0] + g->nbx * (bx[1] + g->nby * bx[2]);
  *cel = ic[0] + NC * (ic[1] + NC * ic[2]);
}

void orc_locate(const orc_mesh* g, long n, const double* x, int32_t* block, int32_t* cell) {
  for (long p = 0; p < n; p++) {
    double xx[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    locate_one(g, xx, block + p, cell + p);
  }
}

/* alpha matrix, Eq. D.3 of Lapenta (2017), pic_mover_boris.cpp:1040-1067 */
static void alpha_matrix(double qdt2m, const double B[3], double alpha[9]) {
  double BB[3][3], P[3], sq = qdt2m * qdt2m;
  for (int i = 0; i < 3; i++) {
    P[i] = -qdt2m * B[i];
    for (int j = 0; j <= i; j++) {
      BB[i][j] = sq * B[i] * B[j];
      BB[j][i] = BB[i][j];
    }
  }
  double c0 = 1.0 / (1.0 + sq * (B[0] * B[0] + B[1] * B[1] + B[2] * B[2]));
  alpha[0] = c0 * (1.0 + BB[0][0]);
  alpha[1] = c0 * (-P[2] + BB[0][1]);
  alpha[2] = c0 * (P[1] + BB[0][2]);
  alpha[3] = c0 * (P[2] + BB[1][0]);
  alpha[4] = c0 * (1.0 + BB[1][1]);
  alpha[5] = c0 * (-P[0] + BB[1][2]);
  alpha[6] = c0 * (-P[1] + BB[2][0]);
  alpha[7] = c0 * (P[0] + BB[2][1]);
  alpha[8] = c0 * (1.0 + BB[2][2]);
}

/* Where the magnetic field the particles see lives: 0 the corners
 * (_PIC_FIELD_SOLVER_B_CORNER_BASED_: the Bc arguments are corner arrays), 1 the
 * cell centres (_PIC_FIELD_SOLVER_B_CENTER_BASED_, the reference's default: the
 * same arguments are cell arrays, B^n for the push and B^{n+1} for the
 * deposit, read by CellCentered::Linear's trilinear stencil). */
static int orc_b_center = 0;
void orc_set_b_center(int on) { orc_b_center = on ? 1 : 0; }

/* B at x from the cell centres: GetTriliniarInterpolationStencil
 * (pic_interpolation_routines.cpp:820-905) -- iLoc in cell units from the
 * block's low face, i0 = -1 below half a cell else (int)(iLoc - 0.5), weight
 * iLoc - (i0 + 0.5), the 8 centres in the stencil's order (i, then j, then k
 * innermost), neighbouring blocks' cells beyond the block (periodic) */
static void centre_b(const orc_mesh* g, const int bxyz[3], const double xmin[3], const double x[3],
                     const double* Bc, double B[3]) {
  int i0[3];
  double w[3];
  for (int d = 0; d < 3; d++) {
    const double loc = (x[d] - xmin[d]) / (NC * g->dx[d]) * NC;
    i0[d] = loc < 0.5 ? -1 : (int)(loc - 0.50);
    w[d] = loc - (i0[d] + 0.5);
  }
  B[0] = B[1] = B[2] = 0.0;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      for (int k = 0; k < 2; k++) {
        const double W = (i ? w[0] : 1.0 - w[0]) * (j ? w[1] : 1.0 - w[1]) * (k ? w[2] : 1.0 - w[2]);
        const long c = cidx(g, bxyz[0] * NC + i0[0] + i, bxyz[1] * NC + i0[1] + j, bxyz[2] * NC + i0[2] + k);
        for (int d = 0; d < 3; d++) B[d] += W * Bc[3 * c + d];
      }
}

/* B at each of n points x[3n] (located in block[n]) from the cell-centred
 * field Bc, by the stencil above (a check of the centre-B restatement) */
void orc_centre_b_at(const orc_mesh* g, long n, const double* x, const int32_t* block,
                     const double* Bc, double* B) {
  for (long p = 0; p < n; p++) {
    int bxyz[3];
    double xmin[3];
    block_geom(g, block[p], bxyz, xmin);
    centre_b(g, bxyz, xmin, x + 3 * p, Bc, B + 3 * p);
  }
}

/* Lapenta2017 (pic_mover_boris.cpp:876-1375) for every particle, followed by
 * the re-binning of the moved particle.  Returns the number of particles that
 * were found outside their block on entry (the reference aborts there). */
long orc_push(const orc_mesh* g, long n, double* x, double* v, const uint8_t* spec,
              int32_t* block, int32_t* cell, const double* E_half, const double* Bc_prev) {
  long nbad = 0;
  for (long p = 0; p < n; p++) {
    if (block[p] < 0) continue;  /* deleted at an open face */
    int bxyz[3], iX[3], nd[8][3];
    double xmin[3], xI[3], vI[3], wt[8], wn[8];
    block_geom(g, block[p], bxyz, xmin);
    for (int d = 0; d < 3; d++) { xI[d] = x[3 * p + d]; vI[d] = v[3 * p + d]; }
    nbad += corner_stencil(xmin, g->dx, xI, wt, wn, nd, iX);
    double E[3] = {0, 0, 0}, B[3] = {0, 0, 0};
    for (int s = 0; s < 8; s++) {
      long c = cidx(g, bxyz[0] * NC + iX[0] + nd[s][0], bxyz[1] * NC + iX[1] + nd[s][1],
                    bxyz[2] * NC + iX[2] + nd[s][2]);
      for (int d = 0; d < 3; d++) {
        E[d] += wn[s] * E_half[3 * c + d];
        if (!orc_b_center) B[d] += wn[s] * Bc_prev[3 * c + d];
      }
    }
    if (orc_b_center) centre_b(g, bxyz, xmin, xI, Bc_prev, B);
    int sp = spec[p];
    double dtT = g->dt;
    double qdtm = g->q[sp] * dtT / g->m[sp];
    double qdt2m = 0.5 * qdtm;
    double alpha[9], vF[3], xF[3];
    alpha_matrix(qdt2m, B, alpha);
    for (int i = 0; i < 3; i++) {
      double vp = 0.0;
      for (int j = 0; j < 3; j++) vp += alpha[3 * i + j] * (vI[j] + qdt2m * E[j]);
      vF[i] = 2.0 * vp - vI[i];
    }
    for (int d = 0; d < 3; d++) xF[d] = xI[d] + dtT * vF[d];
    const int nbd[3] = {g->nbx, g->nby, g->nbz};
    int gone = 0;
    for (int d = 0; d < 3; d++)
      if (((orc_open_axes >> d) & 1) &&
          (xF[d] < g->x0[d] || xF[d] >= g->x0[d] + nbd[d] * NC * g->dx[d]))
        gone = 1;
    if (gone) {
      block[p] = cell[p] = -1;
    } else {
      locate_one(g, xF, block + p, cell + p);
    }
    for (int d = 0; d < 3; d++) { x[3 * p + d] = xF[d]; v[3 * p + d] = vF[d]; }
  }
  return nbad;
}

/* OpenFlow injection (PIC::BC::ExternalBoundary::OpenFlow, src/pic/pic_bc.cpp:
 * 330-420) through one face of an open axis: per boundary cell face a Poisson
 * process in time at CalculateInjectionRate_MaxwellianDistribution (:215) x
 * area / weight, a uniform point on the face, the velocity of
 * InjectMaxwellianDistribution (src/pic/pic_vel_distribution.cpp:49-161),
 * then the Lapenta2017 push for the rest of the step (fields E_half, Bc_prev)
 * and the location (periodic wrap; gone again through an open face -> not
 * kept).  Random numbers: the counter-based stream the device uses (a
 * splitmix64 finaliser over (seed, step, source, face cell, draw)).  Writes up
 * to cap particles (x, v, block, cell); returns how many were kept. */
unsigned long long orc_inj_mix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double orc_inj_uniform(unsigned long long key, unsigned* d) {
  return ((double)(orc_inj_mix(key + ((*d)++)) >> 11) + 0.5) * 1.1102230246251565e-16;
}
/* the stream of face cell (or finest face patch) c of source src at step */
unsigned long long orc_inj_key(unsigned long long seed, unsigned long long step, int src, long c) {
  return orc_inj_mix(orc_inj_mix(orc_inj_mix(seed) ^ step) ^ (((unsigned long long)src << 40) | (unsigned long long)c));
}

/* CalculateInjectionRate_MaxwellianDistribution (pic_bc.cpp:215): particles
 * per unit area and time through a face of outward normal nrm */
double orc_inj_flux(double density, const double drift[3], double vth, const double nrm[3]) {
  const double beta = 1.0 / (sqrt(2.0) * vth);
  double vv = 0.0, vnorm = 0.0;
  for (int d = 0; d < 3; d++) { vv += drift[d] * drift[d]; vnorm += drift[d] * nrm[d]; }
  vv = sqrt(vv);
  const double sq = 1.7724538509055160273, sc = vv * beta;
  if (sc > 10.0 && vnorm < 0.0) return fabs(vnorm) * density;
  if (sc > 10.0 && vnorm > 0.0) return 0.0;
  double aa;
  if (vv > 1.0e-6) {
    const double cc = -vnorm / vv;
    aa = (exp(-sc * sc * cc * cc) + sq * sc * cc * (1.0 + erf(sc * cc))) / (2.0 * sq);
  } else {
    aa = 1.0 / (2.0 * sq);
  }
  return fabs(aa) * density / beta;
}

/* InjectMaxwellianDistribution (pic_vel_distribution.cpp:49, 3D branch):
 * an inward velocity drawn from stream key (draw counter d); 0 when the
 * bounded rejection loops did not finish */
int orc_inj_velocity(unsigned long long key, unsigned* d, const double drift[3], const double nrm[3],
                     double beta, double v[3]) {
  int ok = 0;
  v[0] = v[1] = v[2] = 0.0;
  for (int outer = 0; outer < 64 && !ok; outer++) {
    const double dot = drift[0] * nrm[0] + drift[1] * nrm[1] + drift[2] * nrm[2];
    const double sc = beta * fabs(dot);
    double u = 0.0, acc = 0.0;
    int got = 0;
    for (int tries = 0; tries < 4096 && !got; tries++) {
      if (dot <= 0.0) {
        int q = 0;
        do u = -10.0 + 20.0 * orc_inj_uniform(key, d); while (u + sc <= 0.0 && ++q < 4096);
        const double cc = sqrt(2.0 + sc * sc);
        acc = 2.0 * (u + sc) / (sc + cc) * exp(0.5 + 0.5 * sc * (sc - cc) - u * u);
      } else {
        int q = 0;
        do u = -10.0 + 20.0 * orc_inj_uniform(key, d); while (u + sc >= 0.0 && ++q < 4096);
        const double cc = 0.5 * (-sqrt(sc * sc + 2.0) - sc);
        acc = (u + sc) * exp(-u * u) / (cc + sc) / exp(-cc * cc);
      }
      got = !(acc < orc_inj_uniform(key, d));
    }
    if (!got) break;
    double v1[3], v2[3], v3[3];
    for (int q = 0; q < 3; q++) v3[q] = -(fabs(u + sc) / beta) * nrm[q];
    if (fabs(nrm[0]) > 1.0e-3) { v2[0] = nrm[1]; v2[1] = -nrm[0]; v2[2] = 0.0; }
    else { v2[0] = 0.0; v2[1] = nrm[2]; v2[2] = -nrm[1]; }
    double l2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
    for (int q = 0; q < 3; q++) v2[q] /= l2;
    v1[0] = v2[1] * nrm[2] - v2[2] * nrm[1];
    v1[1] = -(v2[0] * nrm[2] - v2[2] * nrm[0]);
    v1[2] = v2[0] * nrm[1] - v2[1] * nrm[0];
    double l1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
    for (int q = 0; q < 3; q++) v1[q] /= l1;
    const double cm = sqrt(-log(orc_inj_uniform(key, d))) / beta, cp = orc_inj_uniform(key, d);
    const double d1 = drift[0] * v1[0] + drift[1] * v1[1] + drift[2] * v1[2];
    const double d2 = drift[0] * v2[0] + drift[1] * v2[1] + drift[2] * v2[2];
    for (int q = 0; q < 3; q++)
      v[q] = (cm * sin(2.0 * PI_D * cp) + d1) * v1[q] + (cm * cos(2.0 * PI_D * cp) + d2) * v2[q] + v3[q];
    ok = v[0] * nrm[0] + v[1] * nrm[1] + v[2] * nrm[2] < 0.0;
  }
  return ok;
}

long orc_inject(const orc_mesh* g, int face, int spec, double density, const double drift[3],
                double vth, unsigned long long seed, unsigned long long step, int src,
                const double* E_half, const double* Bc_prev, long cap, double* xo, double* vo,
                int32_t* blk, int32_t* cel) {
  const int nb[3] = {g->nbx, g->nby, g->nbz};
  const int ax = face >> 1, hi = face & 1, ta = (ax + 1) % 3, tb = (ax + 2) % 3;
  const double beta = 1.0 / (sqrt(2.0) * vth);
  double nrm[3] = {0, 0, 0};
  nrm[ax] = hi ? 1.0 : -1.0;
  const double flux = orc_inj_flux(density, drift, vth, nrm);
  const double R = (flux / g->w[spec]) * (g->dx[ta] * g->dx[tb]);  /* the device's order */
  const int NT = NC * nb[ta], ncell = NT * NC * nb[tb];
  long kept = 0;
  if (!(R > 0.0)) return 0;
  for (int c = 0; c < ncell; c++) {
    const int it = c % NT, ib = c / NT;
    const unsigned long long key = orc_inj_key(seed, step, src, c);
    unsigned d = 0;
    double tt = 0.0;
    for (int k = 0; k < 4096; k++) {
      tt += -log(orc_inj_uniform(key, &d)) / R;
      if (tt >= g->dt) break;
      const double c0 = orc_inj_uniform(key, &d), c1 = orc_inj_uniform(key, &d);
      double v[3];
      if (!orc_inj_velocity(key, &d, drift, nrm, beta, v)) return -1;
      /* the face point, then the push for the rest of the step */
      double x[3];
      x[ax] = g->x0[ax] + (hi ? nb[ax] * NC * g->dx[ax] : 0.0);
      x[ta] = g->x0[ta] + (it + c0) * g->dx[ta];
      x[tb] = g->x0[tb] + (ib + c1) * g->dx[tb];
      int bxyz[3], iX[3], nd[8][3];
      double xmin[3], wt[8], wn[8], xs[3] = {x[0], x[1], x[2]};
      int bb[3];
      for (int q = 0; q < 3; q++) {
        bb[q] = (int)floor((x[q] - g->x0[q]) / (NC * g->dx[q]));
        if (bb[q] >= nb[q]) bb[q] = nb[q] - 1;
        if (bb[q] < 0) bb[q] = 0;
      }
      block_geom(g, bb[0] + g->nbx * (bb[1] + g->nby * bb[2]), bxyz, xmin);
      corner_stencil(xmin, g->dx, xs, wt, wn, nd, iX);
      double E[3] = {0, 0, 0}, B[3] = {0, 0, 0};
      for (int s = 0; s < 8; s++) {
        long ci = cidx(g, bxyz[0] * NC + iX[0] + nd[s][0], bxyz[1] * NC + iX[1] + nd[s][1],
                       bxyz[2] * NC + iX[2] + nd[s][2]);
        for (int q = 0; q < 3; q++) { E[q] += wn[s] * E_half[3 * ci + q]; B[q] += wn[s] * Bc_prev[3 * ci + q]; }
      }
      const double drem = g->dt - tt;
      const double h = 0.5 * g->q[spec] * drem / g->m[spec];
      double alpha[9], vF[3];
      alpha_matrix(h, B, alpha);
      for (int i = 0; i < 3; i++) {
        double vp = 0.0;
        for (int j = 0; j < 3; j++) vp += alpha[3 * i + j] * (v[j] + h * E[j]);
        vF[i] = 2.0 * vp - v[i];
      }
      for (int q = 0; q < 3; q++) x[q] += drem * vF[q];
      int gone = 0;
      for (int q = 0; q < 3; q++)
        if (((orc_open_axes >> q) & 1) && (x[q] < g->x0[q] || x[q] >= g->x0[q] + nb[q] * NC * g->dx[q]))
          gone = 1;
      if (gone) continue;
      if (kept < cap) {
        locate_one(g, x, blk + kept, cel + kept);
        for (int q = 0; q < 3; q++) { xo[3 * kept + q] = x[q]; vo[3 * kept + q] = vF[q]; }
      }
      kept++;
    }
  }
  return kept;
}

/* Mover::Relativistic::Boris (src/pic/pic_mover_relativistic_boris.cpp:16-583,
 * scalar path :119-175) on the mesh fields: sub-steps of dt = min(1/f_g,
 * remaining) with f_g = |q||B|/(2 pi m gamma) (specfunc.h:1290), fields at the
 * sub-step's start position (corner-interpolated E and B), u = gamma v,
 * u- = u + (q dt/2m) E, t = (q dt/2m / gamma(u-)) B, u' = u- + u- x t,
 * s = 2t/(1+|t|^2), u+ = u- + u' x s, u = u+ + (q dt/2m) E, x += v dt;
 * periodic re-location after every sub-step (findTreeNode).  c = light speed in
 * the mesh's units.  Returns the number of sub-steps. */
long orc_relboris(const orc_mesh* g, long n, double* x, double* v, const uint8_t* spec,
                  int32_t* block, int32_t* cell, const double* E, const double* B, double dt_total,
                  double c_light) {
  long nsub = 0;
  for (long p = 0; p < n; p++) {
    double xI[3], vI[3];
    for (int d = 0; d < 3; d++) { xI[d] = x[3 * p + d]; vI[d] = v[3 * p + d]; }
    const int sp = spec[p];
    const double q = g->q[sp], m = g->m[sp];
    double rem = dt_total;
    while (rem > 0.0) {
      int bxyz[3], iX[3], nd[8][3];
      double xmin[3], wt[8], wn[8], xs[3] = {xI[0], xI[1], xI[2]};
      locate_one(g, xs, block + p, cell + p);
      for (int d = 0; d < 3; d++) xI[d] = xs[d];
      block_geom(g, block[p], bxyz, xmin);
      corner_stencil(xmin, g->dx, xs, wt, wn, nd, iX);
      double Ef[3] = {0, 0, 0}, Bf[3] = {0, 0, 0};
      for (int s2 = 0; s2 < 8; s2++) {
        long c = cidx(g, bxyz[0] * NC + iX[0] + nd[s2][0], bxyz[1] * NC + iX[1] + nd[s2][1],
                      bxyz[2] * NC + iX[2] + nd[s2][2]);
        for (int d = 0; d < 3; d++) {
          Ef[d] += wn[s2] * E[3 * c + d];
          Bf[d] += wn[s2] * B[3 * c + d];
        }
      }
      const double v2 = vI[0] * vI[0] + vI[1] * vI[1] + vI[2] * vI[2];
      double gam = 1.0 / sqrt(1.0 - v2 / (c_light * c_light));
      const double bmag = sqrt(Bf[0] * Bf[0] + Bf[1] * Bf[1] + Bf[2] * Bf[2]);
      double dt = rem;
      if (bmag > 1.0e-25) {
        const double fg = fabs(q) * bmag / (2.0 * PI_D * m * gam);
        const double dtmax = 1.0 / fg;
        if (dtmax < rem) dt = dtmax;
      }
      rem -= dt;
      const double h = q * dt / (2.0 * m);
      double um[3], t[3], up[3], s[3], upl[3], uf[3], l = 0.0;
      for (int d = 0; d < 3; d++) um[d] = gam * vI[d] + h * Ef[d];
      gam = sqrt(1.0 + (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]) / (c_light * c_light));
      for (int d = 0; d < 3; d++) { t[d] = h / gam * Bf[d]; l += t[d] * t[d]; }
      up[0] = um[0] + (um[1] * t[2] - um[2] * t[1]);
      up[1] = um[1] + (um[2] * t[0] - um[0] * t[2]);
      up[2] = um[2] + (um[0] * t[1] - um[1] * t[0]);
      for (int d = 0; d < 3; d++) s[d] = 2.0 * t[d] / (1.0 + l);
      upl[0] = um[0] + (up[1] * s[2] - up[2] * s[1]);
      upl[1] = um[1] + (up[2] * s[0] - up[0] * s[2]);
      upl[2] = um[2] + (up[0] * s[1] - up[1] * s[0]);
      for (int d = 0; d < 3; d++) uf[d] = upl[d] + h * Ef[d];
      gam = sqrt(1.0 + (uf[0] * uf[0] + uf[1] * uf[1] + uf[2] * uf[2]) / (c_light * c_light));
      for (int d = 0; d < 3; d++) {
        vI[d] = uf[d] / gam;
        xI[d] += vI[d] * dt;
      }
      nsub++;
      /* findTreeNode finds no block past an open face: the particle is deleted */
      const int nbd[3] = {g->nbx, g->nby, g->nbz};
      for (int d = 0; d < 3; d++)
        if (((orc_open_axes >> d) & 1) &&
            (xI[d] < g->x0[d] || xI[d] >= g->x0[d] + nbd[d] * NC * g->dx[d]))
          rem = -1.0;
    }
    for (int d = 0; d < 3; d++) { x[3 * p + d] = xI[d]; v[3 * p + d] = vI[d]; }
    if (rem < 0.0) {
      block[p] = cell[p] = -1;
      continue;
    }
    locate_one(g, xI, block + p, cell + p);
    for (int d = 0; d < 3; d++) x[3 * p + d] = xI[d];
  }
  return nsub;
}

/* Mover::Boris (pic_mover_boris.cpp:126-553): one step of dt per particle
 * with E, B interpolated at the start position (CornerBased::InitStencil
 * weights) from the corner arrays (interleaved x, y, z), x' = x + dt v'
 * (:288-290), then findTreeNode/FindCellIndex (periodic wrap; past a face of
 * an open axis the particle is deleted: block = cell = -1).  Returns the
 * number of deleted particles. */
long orc_boris(const orc_mesh* g, long n, double* x, double* v, const uint8_t* spec,
               int32_t* block, int32_t* cell, const double* E, const double* B, double dt) {
  long ndel = 0;
  const int nbd[3] = {g->nbx, g->nby, g->nbz};
  for (long p = 0; p < n; p++) {
    double xs[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    int bxyz[3], iX[3], nd[8][3];
    double xmin[3], wt[8], wn[8];
    locate_one(g, xs, block + p, cell + p);
    block_geom(g, block[p], bxyz, xmin);
    corner_stencil(xmin, g->dx, xs, wt, wn, nd, iX);
    double Ef[3] = {0, 0, 0}, Bf[3] = {0, 0, 0};
    for (int s2 = 0; s2 < 8; s2++) {
      long c = cidx(g, bxyz[0] * NC + iX[0] + nd[s2][0], bxyz[1] * NC + iX[1] + nd[s2][1],
                    bxyz[2] * NC + iX[2] + nd[s2][2]);
      for (int d = 0; d < 3; d++) {
        Ef[d] += wn[s2] * E[3 * c + d];
        Bf[d] += wn[s2] * B[3 * c + d];
      }
    }
    double* vp = v + 3 * p;
    orc_boris_velocity(g->q[spec[p]] / g->m[spec[p]], dt, Ef, Bf, vp);
    int gone = 0;
    for (int d = 0; d < 3; d++) {
      xs[d] = xs[d] + dt * vp[d];
      if (((orc_open_axes >> d) & 1) &&
          (xs[d] < g->x0[d] || xs[d] >= g->x0[d] + nbd[d] * NC * g->dx[d]))
        gone = 1;
    }
    for (int d = 0; d < 3; d++) x[3 * p + d] = xs[d];
    if (gone) {
      block[p] = cell[p] = -1;
      ndel++;
      continue;
    }
    locate_one(g, xs, block + p, cell + p);
    for (int d = 0; d < 3; d++) x[3 * p + d] = xs[d];
  }
  return ndel;
}

/* IndexMatrix[c1][c2] of ProcessCell (pic_field_solver_ecsim.cpp:1889-1891):
 * neighbour slot of corner c2 as seen from corner c1. */
static int index_matrix(int c1, int c2) {
  return slot_of(kCornerOff[c2][0] - kCornerOff[c1][0], kCornerOff[c2][1] - kCornerOff[c1][1],
                 kCornerOff[c2][2] - kCornerOff[c1][2]);
}

/* ProcessCell (pic_field_solver_ecsim.cpp:1882-2438, scalar path) over all
 * cells with the flush of UpdateJMassMatrix (:3244-3995).  J and M are
 * overwritten.  Returns the total particle kinetic energy. */
double orc_deposit(const orc_mesh* g, long n, const double* x, const double* v,
                   const uint8_t* spec, const double* wcorr, const int32_t* block,
                   const int32_t* cell, const double* Bc_cur, double* J, double* M) {
  const long ncell = (long)NC * NC * NC * g->nbx * g->nby * g->nbz;
  double* cJ = (double*)calloc((size_t)ncell * 24, sizeof(double));
  double* cM = (double*)calloc((size_t)ncell * 36 * 9, sizeof(double));
  double V = g->dx[0] * g->dx[1] * g->dx[2];
  double energy = 0.0;
  for (long p = 0; p < n; p++) {
    if (block[p] < 0) continue;
    int bxyz[3], iX[3], nd[8][3];
    double xmin[3], xI[3], vI[3], wt[8], wn[8];
    block_geom(g, block[p], bxyz, xmin);
    for (int d = 0; d < 3; d++) { xI[d] = x[3 * p + d]; vI[d] = v[3 * p + d]; }
    corner_stencil(xmin, g->dx, xI, wt, wn, nd, iX);
    double B[3] = {0, 0, 0};
    if (orc_b_center) {
      centre_b(g, bxyz, xmin, xI, Bc_cur, B);
    } else {
      for (int s = 0; s < 8; s++) {
        long c = cidx(g, bxyz[0] * NC + iX[0] + nd[s][0], bxyz[1] * NC + iX[1] + nd[s][1],
                      bxyz[2] * NC + iX[2] + nd[s][2]);
        for (int d = 0; d < 3; d++) B[d] += wn[s] * Bc_cur[3 * c + d];
      }
    }
    int sp = spec[p];
    double W = g->w[sp] * (wcorr ? wcorr[p] : 1.0);
    double chargeQ = g->q[sp] * W, mass = g->m[sp] * W;
    double qdtm = chargeQ * g->dt / mass, qdt2m = 0.5 * qdtm;
    double alpha[9];
    alpha_matrix(qdt2m, B, alpha);
    double vsqr = vI[0] * vI[0] + vI[1] * vI[1] + vI[2] * vI[2];
    energy += 0.5 * mass * vsqr;
    double vRot[3] = {0, 0, 0};
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) vRot[i] += alpha[3 * i + j] * vI[j];
    long cl = (long)block[p] * 512 + cell[p];
    double* Jg = cJ + cl * 24;
    for (int c = 0; c < 8; c++) {
      double t = chargeQ * wt[c];
      for (int d = 0; d < 3; d++) Jg[3 * c + d] += t * vRot[d];
    }
    double mc = chargeQ * qdt2m / V;
    double* MM = cM + cl * 324;
    int pr = 0;
    for (int c1 = 0; c1 < 8; c1++) {
      double twc = mc * wt[c1];
      for (int c2 = 0; c2 <= c1; c2++, pr++) {
        double twp = wt[c2] * twc;
        for (int ab = 0; ab < 9; ab++) MM[pr * 9 + ab] += alpha[ab] * twp;
      }
    }
  }
  /* flush (ProcessCell :2362-2426 into the shared corner nodes) */
  const long ncor = ncell;
  memset(J, 0, sizeof(double) * 3 * ncor);
  memset(M, 0, sizeof(double) * 243 * ncor);
  for (int b = 0; b < g->nbx * g->nby * g->nbz; b++) {
    int bxyz[3];
    double xmin[3];
    block_geom(g, b, bxyz, xmin);
    for (int lc = 0; lc < 512; lc++) {
      int i = lc % NC, j = (lc / NC) % NC, k = lc / (NC * NC);
      long cl = (long)b * 512 + lc;
      long cor[8];
      for (int c = 0; c < 8; c++)
        cor[c] = cidx(g, bxyz[0] * NC + i + kCornerOff[c][0], bxyz[1] * NC + j + kCornerOff[c][1],
                      bxyz[2] * NC + k + kCornerOff[c][2]);
      for (int c = 0; c < 8; c++)
        for (int d = 0; d < 3; d++) J[3 * cor[c] + d] += cJ[cl * 24 + 3 * c + d] / V;
      int pr = 0;
      for (int c1 = 0; c1 < 8; c1++)
        for (int c2 = 0; c2 <= c1; c2++, pr++) {
          const double* mm = cM + cl * 324 + pr * 9;
          if (c1 == c2) {
            for (int ab = 0; ab < 9; ab++) M[243 * cor[c1] + ab] += mm[ab];
          } else {
            int n12 = index_matrix(c1, c2), n21 = index_matrix(c2, c1);
            for (int ab = 0; ab < 9; ab++) {
              M[243 * cor[c1] + 9 * n12 + ab] += mm[ab];
              M[243 * cor[c2] + 9 * n21 + ab] += mm[ab];
            }
          }
        }
    }
  }
  free(cJ);
  free(cM);
  return energy;
}

/* Per-species maximum over cells of ProcessCell's cflCell
 * (pic_field_solver_ecsim.cpp:2236 sums |v| dt per species, :2356-2359 divides
 * by the count times the cell diagonal; UpdateJMassMatrix keeps the maximum,
 * :3352 and :3972-3977).  A cell without particles of a species gives 0/0 in
 * the reference, which its > test never keeps, so such cells do not count.
 * cfl_max[g->nspec]. */
void orc_cfl(const orc_mesh* g, long n, const double* v, const uint8_t* spec,
             const int32_t* block, const int32_t* cell, double* cfl_max) {
  const long ncell = (long)NC * NC * NC * g->nbx * g->nby * g->nbz;
  const int ns = g->nspec;
  double* sum = (double*)calloc((size_t)ncell * ns, sizeof(double));
  long* cnt = (long*)calloc((size_t)ncell * ns, sizeof(long));
  for (long p = 0; p < n; p++) {
    if (block[p] < 0) continue;
    const long cl = (long)block[p] * 512 + cell[p];
    const double* vp = v + 3 * p;
    const double vsqr = vp[0] * vp[0] + vp[1] * vp[1] + vp[2] * vp[2];
    sum[cl * ns + spec[p]] += sqrt(vsqr) * g->dt;
    cnt[cl * ns + spec[p]] += 1;
  }
  const double diag = sqrt(g->dx[0] * g->dx[0] + g->dx[1] * g->dx[1] + g->dx[2] * g->dx[2]);
  for (int s2 = 0; s2 < ns; s2++) cfl_max[s2] = 0.0;
  for (long c = 0; c < ncell; c++)
    for (int s2 = 0; s2 < ns; s2++)
      if (cnt[c * ns + s2] > 0) {
        const double cf = sum[c * ns + s2] / ((double)cnt[c * ns + s2] * diag);
        if (cf > cfl_max[s2]) cfl_max[s2] = cf;
      }
  free(sum);
  free(cnt);
}

/* Species moments on corners (_PIC_FIELD_SOLVER_SAMPLE_SPECIES_ON_CORNER_,
 * ProcessCell pic_field_solver_ecsim.cpp:2270-2303 and the flush :2384-2394):
 * per particle and corner t = m W w_c, the ten sums rho, rho u (3),
 * rho u u (xx, yy, zz, xy, yz, xz) of its species, divided by the cell volume;
 * out[corner*10*nspec + 10*spec + q] (Rho_ .. RhoUxUz_ order, :138-147). */
void orc_species_moments(const orc_mesh* g, long n, const double* x, const double* v,
                         const uint8_t* spec, const double* wcorr, const int32_t* block,
                         const int32_t* cell, double* out) {
  const long ncor = (long)NC * NC * NC * g->nbx * g->nby * g->nbz;
  const int nq = 10 * g->nspec;
  const double V = g->dx[0] * g->dx[1] * g->dx[2];
  memset(out, 0, sizeof(double) * ncor * nq);
  for (long p = 0; p < n; p++) {
    if (block[p] < 0) continue;
    int bxyz[3], iX[3], nd[8][3];
    double xmin[3], xI[3], wt[8], wn[8];
    block_geom(g, block[p], bxyz, xmin);
    for (int d = 0; d < 3; d++) xI[d] = x[3 * p + d];
    corner_stencil(xmin, g->dx, xI, wt, wn, nd, iX);
    (void)cell;
    const int sp = spec[p];
    const double mass = g->m[sp] * g->w[sp] * (wcorr ? wcorr[p] : 1.0);
    const double* u = v + 3 * p;
    for (int c = 0; c < 8; c++) {
      const long cor = cidx(g, bxyz[0] * NC + iX[0] + kCornerOff[c][0],
                            bxyz[1] * NC + iX[1] + kCornerOff[c][1],
                            bxyz[2] * NC + iX[2] + kCornerOff[c][2]);
      const double t = mass * wt[c], t0 = t * u[0], t1 = t * u[1], t2 = t * u[2];
      double* o = out + cor * nq + 10 * sp;
      o[0] += t / V;
      o[1] += t0 / V;
      o[2] += t1 / V;
      o[3] += t2 / V;
      o[4] += t0 * u[0] / V;
      o[5] += t1 * u[1] / V;
      o[6] += t2 * u[2] / V;
      o[7] += t0 * u[1] / V;
      o[8] += t1 * u[2] / V;
      o[9] += t0 * u[2] / V;
    }
  }
}

/* InterpolateB_C2N (pic_field_solver_ecsim.cpp:5715-5775) */
void orc_center_to_corner(const orc_mesh* g, const double* Bcen, double* Bcor) {
  const int NX = NC * g->nbx, NY = NC * g->nby, NZ = NC * g->nbz;
  for (int K = 0; K < NZ; K++)
    for (int J = 0; J < NY; J++)
      for (int I = 0; I < NX; I++) {
        double t[3] = {0, 0, 0};
        for (int kk = -1; kk <= 0; kk++)
          for (int jj = -1; jj <= 0; jj++)
            for (int ii = -1; ii <= 0; ii++) {
              long c = cidx(g, I + ii, J + jj, K + kk);
              for (int d = 0; d < 3; d++) t[d] += Bcen[3 * c + d];
            }
        long o = cidx(g, I, J, K);
        for (int d = 0; d < 3; d++) Bcor[3 * o + d] = t[d] / 8.0;
      }
}

/* Matrix-free operator: the row assembled by GetStencil and valued by
 * UpdateMatrixElement (pic_field_solver_ecsim.cpp:6004-6019):
 * A = I + (theta c dt)^2 curl curl + 4 pi theta dt M. */
void orc_matvec(const orc_mesh* g, const double* M, const double* x, double* y) {
  const int NX = NC * g->nbx, NY = NC * g->nby, NZ = NC * g->nbz;
  double K[3][3][27];
  operator_taps(g, K, 1);
  const double f = 4.0 * PI_D * g->dt * g->theta;
  for (int Kz = 0; Kz < NZ; Kz++)
    for (int Jy = 0; Jy < NY; Jy++)
      for (int Ix = 0; Ix < NX; Ix++) {
        long c = cidx(g, Ix, Jy, Kz);
        const double* Mc = M + 243 * c;
        for (int p = 0; p < 3; p++) {
          double acc = 0.0;
          for (int dk = -1; dk <= 1; dk++)
            for (int dj = -1; dj <= 1; dj++)
              for (int di = -1; di <= 1; di++) {
                int s = slot_of(di, dj, dk);
                long nb = cidx(g, Ix + di, Jy + dj, Kz + dk);
                for (int q = 0; q < 3; q++)
                  acc += (K[p][q][s] + f * Mc[9 * s + 3 * p + q]) * x[3 * nb + q];
              }
          y[3 * c + p] = acc;
        }
      }
}

void orc_jacobi_diag(const orc_mesh* g, const double* M, double* diag) {
  const long nc = (long)NC * NC * NC * g->nbx * g->nby * g->nbz;
  double K[3][3][27];
  operator_taps(g, K, 1);
  const double f = 4.0 * PI_D * g->dt * g->theta;
  for (long c = 0; c < nc; c++)
    for (int p = 0; p < 3; p++) diag[3 * c + p] = K[p][p][0] + f * M[243 * c + 4 * p];
}

/* UpdateRhs with the supports GetStencil registers (get_stencil.cpp:1260-1599,
 * ecsim/update_rhs.cpp:285-507):
 *   rhs = theta c dt curl B^n - 4 pi theta dt J - (theta c dt)^2 curlcurl E^n
 *         - 4 pi theta dt M E^n */
void orc_rhs(const orc_mesh* g, const double* E_n, const double* Bcen, const double* J,
             const double* M, double* rhs) {
  const int NX = NC * g->nbx, NY = NC * g->nby, NZ = NC * g->nbz;
  double K[3][3][27], c4[3];
  operator_taps(g, K, 0);
  for (int d = 0; d < 3; d++) c4[d] = 0.25 * (g->dt / g->dx[d] * g->theta);
  const double f = 4.0 * PI_D * g->dt * g->theta;
#define BC(ii, jj, kk, comp) Bcen[3 * cidx(g, (ii), (jj), (kk)) + (comp)]
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        long c = cidx(g, i, j, k);
        const double* Mc = M + 243 * c;
        for (int p = 0; p < 3; p++) {
          double res = 0.0;
          for (int dk = -1; dk <= 1; dk++)
            for (int dj = -1; dj <= 1; dj++)
              for (int di = -1; di <= 1; di++) {
                int s = slot_of(di, dj, dk);
                long nb = cidx(g, i + di, j + dj, k + dk);
                for (int q = 0; q < 3; q++)
                  res += (-K[p][q][s] - f * Mc[9 * s + 3 * p + q]) * E_n[3 * nb + q];
              }
          res += -f * J[3 * c + p];
          double cb = 0.0;
          for (int a = -1; a <= 0; a++)
            for (int b = -1; b <= 0; b++) {
              if (p == 0) {
                cb += c4[1] * (BC(i + a, j, k + b, 2) - BC(i + a, j - 1, k + b, 2));
                cb += -c4[2] * (BC(i + a, j + b, k, 1) - BC(i + a, j + b, k - 1, 1));
              } else if (p == 1) {
                cb += c4[2] * (BC(i + a, j + b, k, 0) - BC(i + a, j + b, k - 1, 0));
                cb += -c4[0] * (BC(i, j + b, k + a, 2) - BC(i - 1, j + b, k + a, 2));
              } else {
                cb += c4[0] * (BC(i, j + b, k + a, 1) - BC(i - 1, j + b, k + a, 1));
                cb += -c4[1] * (BC(i + b, j, k + a, 0) - BC(i + b, j - 1, k + a, 0));
              }
            }
          rhs[3 * c + p] = res + cb;
        }
      }
#undef BC
}

static double dot(long n, const double* a, const double* b) {
  double s = 0.0;
  for (long i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* Restarted right-preconditioned GMRES(restart) with modified Gram-Schmidt and
 * Givens rotations.  The reference calls SWMF's linear_solver_wrapper("GMRES",
 * ...) with x0 = 0 (LinearSystemCornerNode.h:3278-3282, absent here); this is
 * the stop rule used throughout: ||b - A x||_2 <= tol ||b||_2.  precond: 0 none,
 * 1 Jacobi.  Returns iterations, or -iterations when not converged. */
int orc_gmres(const orc_mesh* g, const double* M, const double* b, double* x, double tol,
              int maxit, int restart, int precond, double* resid_out) {
  const long n = 3L * NC * NC * NC * g->nbx * g->nby * g->nbz;
  const int m = restart;
  double* V = (double*)malloc(sizeof(double) * n * (m + 1));
  double* Z = (double*)malloc(sizeof(double) * n);
  double* w = (double*)malloc(sizeof(double) * n);
  double* dinv = (double*)malloc(sizeof(double) * n);
  double* H = (double*)calloc((size_t)(m + 1) * m, sizeof(double));
  double *cs = (double*)malloc(sizeof(double) * m), *sn = (double*)malloc(sizeof(double) * m);
  double* s = (double*)malloc(sizeof(double) * (m + 1));
  double* y = (double*)malloc(sizeof(double) * m);
  if (precond) {
    orc_jacobi_diag(g, M, dinv);
    for (long i = 0; i < n; i++) dinv[i] = 1.0 / dinv[i];
  } else {
    for (long i = 0; i < n; i++) dinv[i] = 1.0;
  }
  for (long i = 0; i < n; i++) x[i] = 0.0;
  double bnorm = sqrt(dot(n, b, b));
  int it = 0, conv = 0;
  double rel = 0.0;
  if (bnorm == 0.0) { conv = 1; goto done; }
  while (it < maxit) {
    orc_matvec(g, M, x, w);
    for (long i = 0; i < n; i++) V[i] = b[i] - w[i];
    double beta = sqrt(dot(n, V, V));
    rel = beta / bnorm;
    if (rel <= tol) { conv = 1; break; }
    for (long i = 0; i < n; i++) V[i] /= beta;
    for (int i = 0; i <= m; i++) s[i] = 0.0;
    s[0] = beta;
    int j;
    for (j = 0; j < m && it < maxit; j++) {
      it++;
      for (long i = 0; i < n; i++) Z[i] = dinv[i] * V[j * n + i];
      orc_matvec(g, M, Z, w);
      for (int i = 0; i <= j; i++) {
        double h = dot(n, w, V + i * n);
        H[i * m + j] = h;
        for (long t = 0; t < n; t++) w[t] -= h * V[i * n + t];
      }
      double hn = sqrt(dot(n, w, w));
      H[(j + 1) * m + j] = hn;
      for (long t = 0; t < n; t++) V[(j + 1) * n + t] = (hn > 0.0) ? w[t] / hn : 0.0;
      for (int i = 0; i < j; i++) {
        double a = H[i * m + j], c = H[(i + 1) * m + j];
        H[i * m + j] = cs[i] * a + sn[i] * c;
        H[(i + 1) * m + j] = -sn[i] * a + cs[i] * c;
      }
      double a = H[j * m + j], c = H[(j + 1) * m + j];
      double r = sqrt(a * a + c * c);
      cs[j] = (r > 0.0) ? a / r : 1.0;
      sn[j] = (r > 0.0) ? c / r : 0.0;
      H[j * m + j] = r;
      H[(j + 1) * m + j] = 0.0;
      s[j + 1] = -sn[j] * s[j];
      s[j] = cs[j] * s[j];
      rel = fabs(s[j + 1]) / bnorm;
      if (rel <= tol) { j++; break; }
    }
    for (int i = j - 1; i >= 0; i--) {
      double t = s[i];
      for (int k = i + 1; k < j; k++) t -= H[i * m + k] * y[k];
      y[i] = t / H[i * m + i];
    }
    for (long t = 0; t < n; t++) {
      double acc = 0.0;
      for (int i = 0; i < j; i++) acc += y[i] * V[i * n + t];
      x[t] += dinv[t] * acc;
    }
    if (rel <= tol) {
      orc_matvec(g, M, x, w);
      for (long i = 0; i < n; i++) w[i] = b[i] - w[i];
      rel = sqrt(dot(n, w, w)) / bnorm;
      if (rel <= tol * 10.0) { conv = 1; break; }
    }
  }
done:
  if (resid_out) *resid_out = rel;
  free(V); free(Z); free(w); free(dinv); free(H); free(cs); free(sn); free(s); free(y);
  return conv ? it : -it;
}

/* UpdateB (pic_field_solver_ecsim.cpp:5160-5711, interior cells): B^{n+1} =
 * B^n - c dt curl E^{n+theta} from the 2x2 face averages of the cell's corners. */
void orc_update_b(const orc_mesh* g, const double* E_half, const double* B_n, double* B_np1) {
  const int NX = NC * g->nbx, NY = NC * g->nby, NZ = NC * g->nbz;
  double c4[3];
  for (int d = 0; d < 3; d++) c4[d] = 0.25 * (g->dt / g->dx[d]);
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        double Ex[2][2][2], Ey[2][2][2], Ez[2][2][2];
        for (int kk = 0; kk < 2; kk++)
          for (int jj = 0; jj < 2; jj++)
            for (int ii = 0; ii < 2; ii++) {
              long c = cidx(g, i + ii, j + jj, k + kk);
              Ex[ii][jj][kk] = E_half[3 * c];
              Ey[ii][jj][kk] = E_half[3 * c + 1];
              Ez[ii][jj][kk] = E_half[3 * c + 2];
            }
        double t[3] = {0, 0, 0};
        for (int ii = 0; ii < 2; ii++)
          for (int jj = 0; jj < 2; jj++) {
            t[0] += -c4[1] * (Ez[ii][1][jj] - Ez[ii][0][jj]) + c4[2] * (Ey[ii][jj][1] - Ey[ii][jj][0]);
          }
        for (int ii = 0; ii < 2; ii++)
          for (int jj = 0; jj < 2; jj++) {
            t[1] += -c4[2] * (Ex[ii][jj][1] - Ex[ii][jj][0]) + c4[0] * (Ez[1][ii][jj] - Ez[0][ii][jj]);
          }
        for (int ii = 0; ii < 2; ii++)
          for (int jj = 0; jj < 2; jj++) {
            t[2] += -c4[0] * (Ey[1][ii][jj] - Ey[0][ii][jj]) + c4[1] * (Ex[ii][1][jj] - Ex[ii][0][jj]);
          }
        long o = cidx(g, i, j, k);
        for (int d = 0; d < 3; d++) B_np1[3 * o + d] = B_n[3 * o + d] + t[d];
      }
}

/* UpdateE (pic_field_solver_ecsim.cpp:5909-6001): E^{n+1} = (E^{n+theta} -
 * (1-theta) E^n)/theta in place; returns the wave energy
 * sum over cells of (|E_lowcorner|^2 + |B_center|^2)/(8 pi) * V. */
double orc_update_e(const orc_mesh* g, const double* E_half, double* E_n, const double* B_cen) {
  const long nc = (long)NC * NC * NC * g->nbx * g->nby * g->nbz;
  const double V = g->dx[0] * g->dx[1] * g->dx[2], th = g->theta;
  double sum = 0.0;
  for (long c = 0; c < nc; c++) {
    double e[3];
    for (int d = 0; d < 3; d++) {
      e[d] = (E_half[3 * c + d] - (1.0 - th) * E_n[3 * c + d]) / th;
      E_n[3 * c + d] = e[d];
    }
    const double* B = B_cen + 3 * c;
    sum += ((e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) + (B[0] * B[0] + B[1] * B[1] + B[2] * B[2])) *
           0.125 / PI_D * V;
  }
  return sum;
}

int orc_ecsim_step(const orc_mesh* g, long n, double* x, double* v, const uint8_t* spec,
                   const double* wcorr, int32_t* block, int32_t* cell, double* E_n,
                   double* E_half, double* Bcen, double* Bcor_prev, double* Bcor_cur,
                   double* J, double* M, double tol, int maxit, int precond, double* diag) {
  const long nc = (long)NC * NC * NC * g->nbx * g->nby * g->nbz;
  double* rhs = (double*)malloc(sizeof(double) * 3 * nc);
  double* dE = (double*)malloc(sizeof(double) * 3 * nc);
  double* Bnew = (double*)malloc(sizeof(double) * 3 * nc);
  double resid = 0.0;
  /* ECSIM::TimeStep (:6179-6292) */
  orc_rhs(g, E_n, Bcen, J, M, rhs);
  int it = orc_gmres(g, M, rhs, dE, tol, maxit, 30, precond, &resid);
  for (long i = 0; i < 3 * nc; i++) E_half[i] = E_n[i] + dE[i]; /* ProcessFinalSolution :6311 */
  orc_update_b(g, E_half, Bcen, Bnew);
  /* centre B: Bnew = B^{n+1}, Bcen still B^n until the copy below */
  double* Bold = NULL;
  if (orc_b_center) {
    Bold = (double*)malloc(sizeof(double) * 3 * nc);
    memcpy(Bold, Bcen, sizeof(double) * 3 * nc);
  }
  memcpy(Bcen, Bnew, sizeof(double) * 3 * nc);
  /* corner B: prev <- C2N(B^n) (already there), cur <- C2N(B^{n+1}) */
  memcpy(Bcor_prev, Bcor_cur, sizeof(double) * 3 * nc);
  orc_center_to_corner(g, Bcen, Bcor_cur);
  double wave = orc_update_e(g, E_half, E_n, Bcen);
  /* Mover::MoveParticles with E^{n+theta} and B^n (corner or centre), then
   * UpdateJMassMatrix with B^{n+1} */
  orc_push(g, n, x, v, spec, block, cell, E_half, orc_b_center ? Bold : Bcor_prev);
  double pe = orc_deposit(g, n, x, v, spec, wcorr, block, cell, orc_b_center ? Bcen : Bcor_cur, J, M);
  free(Bold);
  if (diag) { diag[0] = pe; diag[1] = wave; diag[2] = resid; }
  free(rhs); free(dE); free(Bnew);
  return it;
}

/* ------------------------------------------------------------------------
 * Gridless relativistic Boris (GridlessParticleMovers.cpp:781-801), dipole
 * field (DipoleInterface.h:99-126, B = mu0/4pi (3 r (m.r)/r^5 - m/r^3) with
 * the moment fixed by the equatorial surface field), uniform external field,
 * gyro-angle step limiter (CutoffRigidityGridless.cpp:1190-1197).
 * ---------------------------------------------------------------------- */
#define C_LIGHT 299792458.0

void orc_dipole_b(const double x[3], double b_eq, double r_e, const double b_ext[3], double B[3]) {
  double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
  if (r2 <= 0.0) { B[0] = B[1] = B[2] = 0.0; return; }
  double r = sqrt(r2), r3 = r2 * r, r5 = r3 * r2;
  /* moment along +z with mu0/4pi*M = B_eq*R_E^3 (DipoleInterface.h:60-72) */
  double k = b_eq * r_e * r_e * r_e;
  double mdotr = k * x[2];
  B[0] = 3.0 * x[0] * mdotr / r5 + b_ext[0];
  B[1] = 3.0 * x[1] * mdotr / r5 + b_ext[1];
  B[2] = 3.0 * x[2] * mdotr / r5 - k / r3 + b_ext[2];
}

static double gamma_of(const double p[3], double m0) {
  double mc = m0 * C_LIGHT;
  return sqrt(1.0 + (p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) / (mc * mc));
}

long orc_trace(long n, double* x, double* p, int32_t* status, int64_t* steps, double q, double m0,
               double b_eq, double r_e, const double b_ext[3], double r_in, double r_out,
               long max_steps, double dphi_max, double dt_max, int single_precision) {
  long total = 0;
  (void)single_precision;
  for (long i = 0; i < n; i++) {
    double* xi = x + 3 * i;
    double* pi = p + 3 * i;
    long s = 0;
    int st = 0;
    while (s < max_steps) {
      double B[3];
      orc_dipole_b(xi, b_eq, r_e, b_ext, B);
      double Bm = sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
      double gam = gamma_of(pi, m0);
      double dt = dt_max;
      if (Bm > 0.0) {
        double om = fabs(q) * Bm / (gam * m0);
        if (om > 0.0 && dphi_max / om < dt) dt = dphi_max / om;
      }
      /* BorisStep: half drift, rotation with B at the start point, half drift */
      double vv = 1.0 / (gam * m0);
      for (int d = 0; d < 3; d++) xi[d] += 0.5 * dt * vv * pi[d];
      double t[3], f = (q * dt) / (2.0 * gam * m0);
      for (int d = 0; d < 3; d++) t[d] = f * B[d];
      double t2 = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
      double sfac = 2.0 / (1.0 + t2);
      double pm[3] = {pi[0], pi[1], pi[2]};
      double pp[3] = {pm[0] + (pm[1] * t[2] - pm[2] * t[1]), pm[1] + (pm[2] * t[0] - pm[0] * t[2]),
                      pm[2] + (pm[0] * t[1] - pm[1] * t[0])};
      double sv[3] = {sfac * t[0], sfac * t[1], sfac * t[2]};
      pi[0] = pm[0] + (pp[1] * sv[2] - pp[2] * sv[1]);
      pi[1] = pm[1] + (pp[2] * sv[0] - pp[0] * sv[2]);
      pi[2] = pm[2] + (pp[0] * sv[1] - pp[1] * sv[0]);
      double g2 = gamma_of(pi, m0);
      double v2 = 1.0 / (g2 * m0);
      for (int d = 0; d < 3; d++) xi[d] += 0.5 * dt * v2 * pi[d];
      s++;
      double r = sqrt(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]);
      if (r < r_in) { st = 1; break; }
      if (r > r_out) { st = 2; break; }
    }
    status[i] = st;
    steps[i] = s;
    total += s;
  }
  return total;
}

/* ===========================================================================
 * Restart particle section and its checksum
 * ======================================================================== */

/* CRC32::generare_crc_table (specfunc.h:449-459): the remainder of each byte
 * value placed in bits 24..31, in a 64-bit word that keeps the bits the eight
 * shifts move above bit 31. */
void orc_crc32_table(uint64_t t[256]) {
  for (int i = 0; i < 256; i++) {
    uint64_t a = (uint64_t)i << 24;
    for (int j = 0; j < 8; j++) a = (a & 0x80000000ull) ? (a << 1) ^ 0x04c11db7ull : a << 1;
    t[i] = a;
  }
}

/* CRC32::add (specfunc.h:471-480): index = bits 24..31 of the accumulator xor
 * the byte; accumulator = (accumulator << 8) xor table[index], all 64 bits. */
uint64_t orc_crc32_add(uint64_t acc, const uint8_t* p, long n) {
  uint64_t t[256];
  orc_crc32_table(t);
  for (long q = 0; q < n; q++) acc = (acc << 8) ^ t[((acc >> 24) ^ p[q]) & 0xffu];
  return acc;
}

/* one record: links (bytes 0..15) and every field the path does not hold are
 * zero (GetParticleSignature with IncludeListInfo=false clones the particle
 * into a zeroed buffer keeping its zero links, pic_pbuffer.cpp:1109-1123) */
static void orc_record(const orc_record_layout* L, const double* x, const double* v, uint8_t sp,
                       double w, uint8_t* rec) {
  memset(rec, 0, (size_t)L->len);
  memcpy(rec + L->off_v, v, 24);
  memcpy(rec + L->off_x, x, 24);
  rec[L->off_sp] = sp;
  if (L->off_w >= 0) memcpy(rec + L->off_w, &w, 8);
}

/* particles grouped by block (in file order) and reference cell order
 * (i slowest, i.e. ParticleNumberTable[i][j][k]); stable, so each cell keeps
 * its list order.  Returns the permutation; start[] gets the group offsets of
 * the nb*512 (block position, i, j, k) groups. */
static long* orc_group(int nb, const int32_t* block_order, long n, const int32_t* block,
                       const int32_t* cell, long** start_out) {
  int* pos = (int*)malloc(sizeof(int) * (size_t)nb);
  for (int q = 0; q < nb; q++) pos[block_order ? block_order[q] : q] = q;
  const long ng = (long)nb * 512;
  long* start = (long*)calloc((size_t)ng + 1, sizeof(long));
  long* key = (long*)malloc(sizeof(long) * (size_t)(n > 0 ? n : 1));
  for (long p = 0; p < n; p++) {
    const int l = cell[p], i = l % 8, j = (l / 8) % 8, k = l / 64;
    key[p] = (long)pos[block[p]] * 512 + i * 64 + j * 8 + k;
    start[key[p] + 1]++;
  }
  for (long g = 0; g < ng; g++) start[g + 1] += start[g];
  long* fill = (long*)malloc(sizeof(long) * (size_t)ng);
  memcpy(fill, start, sizeof(long) * (size_t)ng);
  long* perm = (long*)malloc(sizeof(long) * (size_t)(n > 0 ? n : 1));
  for (long p = 0; p < n; p++) perm[fill[key[p]]++] = p;
  free(fill);
  free(key);
  free(pos);
  *start_out = start;
  return perm;
}

/* PIC::Restart::SaveParticleData / SaveParticleDataBlock (pic_restart.cpp:
 * 248-382): marker, ParticleDataLength, GlobalParticleWeight; per block with
 * particles its node id, count and ParticleNumberTable, then the records of
 * each cell from the list tail to its head (:352-371). */
long long orc_restart_pack(const orc_record_layout* L, int nb, const int32_t* block_order,
                           const uint8_t* node_ids, int id_len, int nspec, const double* weight,
                           long n, const double* x, const double* v, const uint8_t* spec,
                           const double* wcorr, const int32_t* block, const int32_t* cell,
                           uint8_t* out, long long cap) {
  static const char marker[43] = "PARTICLE-RESTART-FILE--END-USER-ADDITIONAL";
  long* start;
  long* perm = orc_group(nb, block_order, n, block, cell, &start);
  long long size = 43 + 8 + 8LL * nspec;
  for (int q = 0; q < nb; q++) {
    const long tot = start[(long)(q + 1) * 512] - start[(long)q * 512];
    if (tot) size += id_len + 4 + 4 * 512 + tot * (long long)L->len;
  }
  if (out && cap < size) {
    free(perm);
    free(start);
    return -1;
  }
  if (out) {
    long long o = 0;
    const long long len = L->len;
    memcpy(out, marker, 43);
    memcpy(out + 43, &len, 8);
    memcpy(out + 51, weight, 8 * (size_t)nspec);
    o = 51 + 8LL * nspec;
    for (int q = 0; q < nb; q++) {
      const long g0 = (long)q * 512;
      const int tot = (int)(start[g0 + 512] - start[g0]);
      if (!tot) continue;
      const int b = block_order ? block_order[q] : q;
      if (id_len) memcpy(out + o, node_ids + (size_t)b * id_len, (size_t)id_len);
      o += id_len;
      memcpy(out + o, &tot, 4);
      o += 4;
      for (int t = 0; t < 512; t++) {
        const int c = (int)(start[g0 + t + 1] - start[g0 + t]);
        memcpy(out + o + 4 * t, &c, 4);
      }
      o += 4 * 512;
      for (int t = 0; t < 512; t++)
        for (long r = start[g0 + t + 1] - 1; r >= start[g0 + t]; r--) {
          const long p = perm[r];
          orc_record(L, x + 3 * p, v + 3 * p, spec[p], wcorr ? wcorr[p] : 1.0, out + o);
          o += L->len;
        }
    }
  }
  free(perm);
  free(start);
  return size;
}

/* PIC::Restart::GetParticleDataCheckSum (pic_restart.cpp:578-660): one CRC32
 * object over the blocks in tree order, cells i, j, k, each list head to tail */
uint64_t orc_particle_checksum(const orc_record_layout* L, int nb, const int32_t* block_order, long n,
                               const double* x, const double* v, const uint8_t* spec,
                               const double* wcorr, const int32_t* block, const int32_t* cell) {
  long* start;
  long* perm = orc_group(nb, block_order, n, block, cell, &start);
  uint64_t t[256];
  orc_crc32_table(t);
  uint8_t rec[512];
  uint64_t acc = 0;
  for (long r = 0; r < n; r++) {
    const long p = perm[r];
    orc_record(L, x + 3 * p, v + 3 * p, spec[p], wcorr ? wcorr[p] : 1.0, rec);
    for (int q = 0; q < L->len; q++) acc = (acc << 8) ^ t[((acc >> 24) ^ rec[q]) & 0xffu];
  }
  free(perm);
  free(start);
  return acc;
}
