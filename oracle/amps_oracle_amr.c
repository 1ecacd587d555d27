/*
 * amps_oracle_amr.c -- FP64 CPU restatement of the ECSIM particle / field path
 * on block-structured AMR meshes.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference's ECSIM discretisation is written corner by corner for a
 * uniform mesh; per cell it is
 *   curl E (cell) = C E_corners     UpdateB, pic_field_solver_ecsim.cpp:5160-5711
 *   curl B (corner) = C^T B_cells   GetStencil's curl B supports, get_stencil.cpp:1500-1599
 *   curl curl = C^T C assembled     the compact stencils of InitDiscritizationStencil :7121
 *   M = per-cell pair sums          ProcessCell, :1882-2438
 * (C: 3 x 24 face-average differences, coefficient 1/(4 dx)).  On an AMR mesh
 * the same per-cell pieces are assembled with each cell's own dx in weak form
 * (every cell term times its volume), and the corners of fine blocks that lie
 * on a coarser block's face or edge without being its corners ("hanging")
 * take the multilinear interpolation of the coarse corners: the operator is
 * P^T A P on the free corners, and hanging rows read x_h - (P x)_h = 0.  On a
 * uniform mesh this is the reference's operator times the cell volume.
 * The reference itself defines no coarse/fine interface (its stencils assume
 * same-level neighbours, get_stencil.cpp:1100-1160): parity across levels is
 * pinned by energy conservation, not by reference output.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "amps_oracle.h"

#define PI_D 3.14159265358979323846264338327950288

extern int orc_open_axes; /* amps_oracle.c */
/* injection helpers (amps_oracle.c) */
unsigned long long orc_inj_key(unsigned long long seed, unsigned long long step, int src, long c);
double orc_inj_uniform(unsigned long long key, unsigned* d);
double orc_inj_flux(double density, const double drift[3], double vth, const double nrm[3]);
int orc_inj_velocity(unsigned long long key, unsigned* d, const double drift[3], const double nrm[3],
                     double beta, double v[3]);
#define NSPEC_MAX 8

typedef struct {
  int nblocks, ncorners, lmax;
  int nfine[3];
  double x0[3], dx0;
  const int32_t* level;       /* nblocks */
  const int32_t* origin;      /* nblocks*3, finest-cell units */
  const int32_t* corner_tab;  /* nblocks*729 */
  const int32_t* hang_start;  /* ncorners+1 */
  const int32_t* hang_parent;
  const double* hang_weight;
  const int32_t* fine_map;    /* finest blocks */
  int nspec;
  double q[NSPEC_MAX], m[NSPEC_MAX], w[NSPEC_MAX];
  double dt, theta;
  /* open (non-periodic) axes: boundary constraint rows of the field solve and
   * UpdateB's boundary branch (NULL flag: fully periodic) */
  const int32_t* bnd_flag;    /* ncorners */
  const int32_t* bnd_start;   /* ncorners+1 */
  const int32_t* bnd_col;
  const double* bnd_weight;
  int open_mask;              /* bit d: axis d open */
  int field_bc;               /* bit 2d + high: Neumann face of open axis d (else Dirichlet) */
} orc_amr;

static const int kOff[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                               {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};



static double bdx(const orc_amr* g, int b) { return g->dx0 / (double)(1 << g->level[b]); }

static void borigin(const orc_amr* g, int b, double o[3]) {
  const double dxf = g->dx0 / (double)(1 << g->lmax);
  for (int d = 0; d < 3; d++) o[d] = g->x0[d] + g->origin[3 * b + d] * dxf;
}

/* value of a corner field (3 comps) with the hanging constraint applied */
static void corner_val(const orc_amr* g, const double* F, int c, double out[3]) {
  const int s = g->hang_start[c], e = g->hang_start[c + 1];
  if (s == e) {
    for (int d = 0; d < 3; d++) out[d] = F[3 * c + d];
    return;
  }
  out[0] = out[1] = out[2] = 0.0;
  for (int t = s; t < e; t++)
    for (int d = 0; d < 3; d++) out[d] += g->hang_weight[t] * F[3 * g->hang_parent[t] + d];
}

static int cell_corner(const orc_amr* g, int b, int i, int j, int k) {
  return g->corner_tab[b * 729 + i + 9 * (j + 9 * k)];
}

/* block containing x (finest-block map), block-local cell (FindCellIndex) */
static void locate_one(const orc_amr* g, double x[3], int32_t* blk, int32_t* cel) {
  const double dxf = g->dx0 / (double)(1 << g->lmax);
  int F[3];
  for (int d = 0; d < 3; d++) {
    const double L = g->nfine[d] * dxf;
    /* periodic wrap of the position itself */
    if (x[d] < g->x0[d]) x[d] += L;
    if (x[d] >= g->x0[d] + L) x[d] -= L;
    if (x[d] >= g->x0[d] + L) x[d] = g->x0[d] + L - 1e-10 * dxf;
    if (x[d] < g->x0[d]) x[d] = g->x0[d];
    F[d] = (int)floor((x[d] - g->x0[d]) / dxf);
    if (F[d] >= g->nfine[d]) F[d] = g->nfine[d] - 1;
    if (F[d] < 0) F[d] = 0;
  }
  const int nfb0 = g->nfine[0] / 8, nfb1 = g->nfine[1] / 8;
  const int b = g->fine_map[F[0] / 8 + nfb0 * (F[1] / 8 + nfb1 * (F[2] / 8))];
  double o[3];
  borigin(g, b, o);
  const double dx = bdx(g, b);
  int ic[3];
  for (int d = 0; d < 3; d++) {
    int i = (int)((x[d] - o[d]) / dx);
    if (i >= 8) i = 7;
    if (i < 0) i = 0;
    ic[d] = i;
  }
  *blk = b;
  *cel = ic[0] + 8 * (ic[1] + 8 * ic[2]);
}

void orc_amr_locate(const orc_amr* g, long n, double* x, int32_t* block, int32_t* cell) {
  for (long p = 0; p < n; p++) locate_one(g, x + 3 * p, block + p, cell + p);
}

static void alpha_matrix(double h, const double B[3], double al[9]) {
  double sq = h * h, P[3], BB[3][3];
  for (int i = 0; i < 3; i++) {
    P[i] = -h * B[i];
    for (int j = 0; j < 3; j++) BB[i][j] = sq * B[i] * B[j];
  }
  double c0 = 1.0 / (1.0 + sq * (B[0] * B[0] + B[1] * B[1] + B[2] * B[2]));
  al[0] = c0 * (1.0 + BB[0][0]); al[1] = c0 * (-P[2] + BB[0][1]); al[2] = c0 * (P[1] + BB[0][2]);
  al[3] = c0 * (P[2] + BB[1][0]); al[4] = c0 * (1.0 + BB[1][1]); al[5] = c0 * (-P[0] + BB[1][2]);
  al[6] = c0 * (-P[1] + BB[2][0]); al[7] = c0 * (P[0] + BB[2][1]); al[8] = c0 * (1.0 + BB[2][2]);
}

/* trilinear weights in table order and the corresponding unique corners */
static void stencil(const orc_amr* g, int b, const double x[3], double w[8], int cid[8]) {
  double o[3], f[3];
  int ic[3];
  borigin(g, b, o);
  const double dx = bdx(g, b);
  for (int d = 0; d < 3; d++) {
    double u = (x[d] - o[d]) / dx;
    int i = (int)u;
    if (i > 7) i = 7;
    if (i < 0) i = 0;
    ic[d] = i;
    f[d] = u - i;
  }
  for (int c = 0; c < 8; c++) {
    double ww = 1.0;
    for (int d = 0; d < 3; d++) ww *= kOff[c][d] ? f[d] : 1.0 - f[d];
    w[c] = ww;
    cid[c] = cell_corner(g, b, ic[0] + kOff[c][0], ic[1] + kOff[c][1], ic[2] + kOff[c][2]);
  }
}

long orc_amr_push(const orc_amr* g, long n, double* x, double* v, const uint8_t* spec,
                  int32_t* block, int32_t* cell, const double* E_half, const double* Bc_prev) {
  const double dxf = g->dx0 / (double)(1 << g->lmax);
  for (long p = 0; p < n; p++) {
    if (block[p] < 0) continue; /* deleted at an open face */
    double w[8], E[3] = {0, 0, 0}, B[3] = {0, 0, 0}, val[3];
    int cid[8];
    stencil(g, block[p], x + 3 * p, w, cid);
    for (int c = 0; c < 8; c++) {
      corner_val(g, E_half, cid[c], val);
      for (int d = 0; d < 3; d++) E[d] += w[c] * val[d];
      corner_val(g, Bc_prev, cid[c], val);
      for (int d = 0; d < 3; d++) B[d] += w[c] * val[d];
    }
    const int s = spec[p];
    const double h = 0.5 * g->q[s] * g->dt / g->m[s];
    double al[9], vn[3];
    alpha_matrix(h, B, al);
    for (int i = 0; i < 3; i++) {
      double vp = 0.0;
      for (int j = 0; j < 3; j++) vp += al[3 * i + j] * (v[3 * p + j] + h * E[j]);
      vn[i] = 2.0 * vp - v[3 * p + i];
    }
    int gone = 0;
    for (int d = 0; d < 3; d++) {
      v[3 * p + d] = vn[d];
      x[3 * p + d] += g->dt * vn[d];
      if (((orc_open_axes >> d) & 1) &&
          (x[3 * p + d] < g->x0[d] || x[3 * p + d] >= g->x0[d] + g->nfine[d] * dxf))
        gone = 1;
    }
    if (gone)
      block[p] = cell[p] = -1;
    else
      locate_one(g, x + 3 * p, block + p, cell + p);
  }
  return 0;
}

/* Mover::Relativistic::Boris (src/pic/pic_mover_relativistic_boris.cpp:16-583,
 * scalar path :119-175) on a periodic AMR mesh: the sub-step rule and the
 * two-rotation update of the uniform-mesh restatement (orc_relboris); at the
 * start of every sub-step the particle is re-located in the block tree
 * (findTreeNode: periodic wrap and the finest-block map) and E, B are the
 * trilinear interpolation from that leaf block's 8 cell corners, hanging
 * corners through their constraint.  E = E^n, B = the corner B of the "cur"
 * slot (interleaved x, y, z per corner).  Returns the number of sub-steps. */
/* a sub-step can carry a fast particle more than one period: shift by whole
 * periods first (the uniform mesh's block-periodic shift), then locate_one */
static void wrap_far(const orc_amr* g, double x[3]) {
  const double dxf = g->dx0 / (double)(1 << g->lmax);
  for (int d = 0; d < 3; d++) {
    const double L = g->nfine[d] * dxf;
    const double k = floor((x[d] - g->x0[d]) / L);
    if (k != 0.0) x[d] -= k * L;
  }
}

long orc_amr_relboris(const orc_amr* g, long n, double* x, double* v, const uint8_t* spec,
                      int32_t* block, int32_t* cell, const double* E, const double* B,
                      double dt_total, double c_light) {
  const double cc2 = c_light * c_light;
  long nsub = 0;
  for (long p = 0; p < n; p++) {
    double* xp = x + 3 * p;
    double* vp = v + 3 * p;
    const int sp = spec[p];
    const double q = g->q[sp], m = g->m[sp];
    double rem = dt_total;
    while (rem > 0.0) {
      double w[8], Ef[3] = {0, 0, 0}, Bf[3] = {0, 0, 0}, val[3];
      int cid[8];
      wrap_far(g, xp);
      locate_one(g, xp, block + p, cell + p);
      stencil(g, block[p], xp, w, cid);
      for (int c = 0; c < 8; c++) {
        corner_val(g, E, cid[c], val);
        for (int d = 0; d < 3; d++) Ef[d] += w[c] * val[d];
        corner_val(g, B, cid[c], val);
        for (int d = 0; d < 3; d++) Bf[d] += w[c] * val[d];
      }
      double gam = 1.0 / sqrt(1.0 - (vp[0] * vp[0] + vp[1] * vp[1] + vp[2] * vp[2]) / cc2);
      const double bmag = sqrt(Bf[0] * Bf[0] + Bf[1] * Bf[1] + Bf[2] * Bf[2]);
      double dt = rem;
      if (bmag > 1.0e-25) {
        const double dtmax = 1.0 / (fabs(q) * bmag / (2.0 * PI_D * m * gam));
        if (dtmax < rem) dt = dtmax;
      }
      rem -= dt;
      const double h = q * dt / (2.0 * m);
      double um[3], t[3], up[3], s[3], upl[3], uf[3], l = 0.0;
      for (int d = 0; d < 3; d++) um[d] = gam * vp[d] + h * Ef[d];
      gam = sqrt(1.0 + (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]) / cc2);
      for (int d = 0; d < 3; d++) {
        t[d] = h / gam * Bf[d];
        l += t[d] * t[d];
      }
      up[0] = um[0] + (um[1] * t[2] - um[2] * t[1]);
      up[1] = um[1] + (um[2] * t[0] - um[0] * t[2]);
      up[2] = um[2] + (um[0] * t[1] - um[1] * t[0]);
      for (int d = 0; d < 3; d++) s[d] = 2.0 * t[d] / (1.0 + l);
      upl[0] = um[0] + (up[1] * s[2] - up[2] * s[1]);
      upl[1] = um[1] + (up[2] * s[0] - up[0] * s[2]);
      upl[2] = um[2] + (up[0] * s[1] - up[1] * s[0]);
      for (int d = 0; d < 3; d++) uf[d] = upl[d] + h * Ef[d];
      gam = sqrt(1.0 + (uf[0] * uf[0] + uf[1] * uf[1] + uf[2] * uf[2]) / cc2);
      for (int d = 0; d < 3; d++) {
        vp[d] = uf[d] / gam;
        xp[d] += vp[d] * dt;
      }
      nsub++;
      /* findTreeNode finds no block past an open face: the particle is deleted */
      for (int d = 0; d < 3; d++)
        if (((orc_open_axes >> d) & 1) &&
            (xp[d] < g->x0[d] || xp[d] >= g->x0[d] + g->nfine[d] * (g->dx0 / (double)(1 << g->lmax))))
          rem = -1.0;
    }
    if (rem < 0.0) {
      block[p] = cell[p] = -1;
      continue;
    }
    wrap_far(g, xp);
    locate_one(g, xp, block + p, cell + p);
  }
  return nsub;
}

/* Mover::Boris (src/pic/pic_mover_boris.cpp:126-553) on a periodic AMR mesh:
 * one step of dt with E, B interpolated at the start position from its leaf
 * block's 8 cell corners (hanging corners through their constraint), the
 * velocity update of orc_boris_velocity, x' = x + dt v', then re-location in
 * the block tree (past a face of an open axis: deleted, block = cell = -1).
 * Returns the number of deleted particles. */
long orc_amr_boris(const orc_amr* g, long n, double* x, double* v, const uint8_t* spec,
                   int32_t* block, int32_t* cell, const double* E, const double* B, double dt) {
  long ndel = 0;
  const double dxf = g->dx0 / (double)(1 << g->lmax);
  for (long p = 0; p < n; p++) {
    double* xp = x + 3 * p;
    double* vp = v + 3 * p;
    double w[8], Ef[3] = {0, 0, 0}, Bf[3] = {0, 0, 0}, val[3];
    int cid[8];
    wrap_far(g, xp);
    locate_one(g, xp, block + p, cell + p);
    stencil(g, block[p], xp, w, cid);
    for (int c = 0; c < 8; c++) {
      corner_val(g, E, cid[c], val);
      for (int d = 0; d < 3; d++) Ef[d] += w[c] * val[d];
      corner_val(g, B, cid[c], val);
      for (int d = 0; d < 3; d++) Bf[d] += w[c] * val[d];
    }
    orc_boris_velocity(g->q[spec[p]] / g->m[spec[p]], dt, Ef, Bf, vp);
    int gone = 0;
    for (int d = 0; d < 3; d++) {
      xp[d] = xp[d] + dt * vp[d];
      if (((orc_open_axes >> d) & 1) && (xp[d] < g->x0[d] || xp[d] >= g->x0[d] + g->nfine[d] * dxf))
        gone = 1;
    }
    if (gone) {
      block[p] = cell[p] = -1;
      ndel++;
      continue;
    }
    wrap_far(g, xp);
    locate_one(g, xp, block + p, cell + p);
  }
  return ndel;
}

/* OpenFlow injection through face `face` of an open axis on the AMR mesh
 * (pic_bc.cpp:270-440 with CalculateInjectionRate_MaxwellianDistribution :215
 * and InjectMaxwellianDistribution, pic_vel_distribution.cpp:49): the face is
 * cut into finest-lattice patches (patch c = it + nfine[ta] ib), each with its
 * own Poisson stream (the device's key); an arrival at time tt is placed
 * uniformly on its patch, pushed with Lapenta2017 for dt - tt with the fields
 * of the leaf block owning the patch's boundary cell, and kept when it stays
 * in the domain.  Returns the kept count (-1: sampling bound hit). */
long orc_amr_inject(const orc_amr* g, int face, int spec, double density, const double drift[3],
                    double vth, unsigned long long seed, unsigned long long step, int src,
                    const double* E_half, const double* Bc_prev, long cap, double* xo, double* vo,
                    int32_t* blk, int32_t* cel) {
  const int ax = face >> 1, hi = face & 1, ta = (ax + 1) % 3, tb = (ax + 2) % 3;
  const double dxf = g->dx0 / (double)(1 << g->lmax);
  const double beta = 1.0 / (sqrt(2.0) * vth);
  double nrm[3] = {0, 0, 0};
  nrm[ax] = hi ? 1.0 : -1.0;
  const double flux = orc_inj_flux(density, drift, vth, nrm);
  const double R = (flux / g->w[spec]) * (dxf * dxf);  /* the device's order */
  const int NT = g->nfine[ta], np = NT * g->nfine[tb];
  long kept = 0;
  if (!(R > 0.0)) return 0;
  for (int c = 0; c < np; c++) {
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
      /* the face point and the leaf block owning the patch's boundary cell */
      int F[3];
      F[ax] = hi ? g->nfine[ax] - 1 : 0;
      F[ta] = it;
      F[tb] = ib;
      const int nfb0 = g->nfine[0] / 8, nfb1 = g->nfine[1] / 8;
      const int b = g->fine_map[F[0] / 8 + nfb0 * (F[1] / 8 + nfb1 * (F[2] / 8))];
      double x[3];
      x[ax] = g->x0[ax] + (hi ? g->nfine[ax] * dxf : 0.0);
      x[ta] = g->x0[ta] + (it + c0) * dxf;
      x[tb] = g->x0[tb] + (ib + c1) * dxf;
      double w[8], E[3] = {0, 0, 0}, B[3] = {0, 0, 0}, val[3], xs[3] = {x[0], x[1], x[2]};
      int cid[8];
      stencil(g, b, xs, w, cid);
      for (int q = 0; q < 8; q++) {
        corner_val(g, E_half, cid[q], val);
        for (int e = 0; e < 3; e++) E[e] += w[q] * val[e];
        corner_val(g, Bc_prev, cid[q], val);
        for (int e = 0; e < 3; e++) B[e] += w[q] * val[e];
      }
      const double drem = g->dt - tt;
      const double h = 0.5 * g->q[spec] * drem / g->m[spec];
      double al[9], vF[3];
      alpha_matrix(h, B, al);
      for (int i = 0; i < 3; i++) {
        double vp = 0.0;
        for (int j = 0; j < 3; j++) vp += al[3 * i + j] * (v[j] + h * E[j]);
        vF[i] = 2.0 * vp - v[i];
      }
      int gone = 0;
      for (int q = 0; q < 3; q++) {
        x[q] += drem * vF[q];
        if (((orc_open_axes >> q) & 1) && (x[q] < g->x0[q] || x[q] >= g->x0[q] + g->nfine[q] * dxf)) gone = 1;
      }
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

/* per-cell partials (cellJ[ncell*24] = sum q W w_c alpha v; cellM[ncell*324] =
 * sum (q W qdt/2m / V) w_c1 w_c2 alpha over pairs c2<=c1).  Returns energy. */
/* ProcessCell's per-particle terms (pic_field_solver_ecsim.cpp:2186-2342) of
 * particle p added to its cell's blocks; returns its kinetic energy. */
static double deposit_one(const orc_amr* g, long p, const double* x, const double* v,
                          const uint8_t* spec, const double* wcorr, const int32_t* block,
                          const int32_t* cell, const double* Bc_cur, double* cellJ, double* cellM) {
  double w[8], B[3] = {0, 0, 0}, val[3];
  int cid[8];
  const int b = block[p];
  stencil(g, b, x + 3 * p, w, cid);
  for (int c = 0; c < 8; c++) {
    corner_val(g, Bc_cur, cid[c], val);
    for (int d = 0; d < 3; d++) B[d] += w[c] * val[d];
  }
  const double dx = bdx(g, b), V = dx * dx * dx;
  const int s = spec[p];
  const double W = g->w[s] * (wcorr ? wcorr[p] : 1.0);
  const double qW = g->q[s] * W, mW = g->m[s] * W;
  const double h = 0.5 * qW * g->dt / mW;
  double al[9], vr[3] = {0, 0, 0};
  alpha_matrix(h, B, al);
  const double* vv = v + 3 * p;
  const double e = 0.5 * mW * (vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) vr[i] += al[3 * i + j] * vv[j];
  const long cl = (long)b * 512 + cell[p];
  for (int c = 0; c < 8; c++)
    for (int d = 0; d < 3; d++) cellJ[cl * 24 + 3 * c + d] += qW * w[c] * vr[d];
  const double mc = qW * h / V;
  int pr = 0;
  for (int c1 = 0; c1 < 8; c1++)
    for (int c2 = 0; c2 <= c1; c2++, pr++)
      for (int ab = 0; ab < 9; ab++) cellM[cl * 324 + pr * 9 + ab] += mc * w[c1] * w[c2] * al[ab];
  return e;
}

double orc_amr_deposit(const orc_amr* g, long n, const double* x, const double* v,
                       const uint8_t* spec, const double* wcorr, const int32_t* block,
                       const int32_t* cell, const double* Bc_cur, double* cellJ, double* cellM) {
  const long ncell = (long)g->nblocks * 512;
  memset(cellJ, 0, sizeof(double) * ncell * 24);
  memset(cellM, 0, sizeof(double) * ncell * 324);
  double energy = 0.0;
  for (long p = 0; p < n; p++) {
    if (block[p] < 0) continue;
    energy += deposit_one(g, p, x, v, spec, wcorr, block, cell, Bc_cur, cellJ, cellM);
  }
  return energy;
}

/* The same push + deposit on nthreads host threads (the reference's HYBRID
 * OpenMP mode runs its mover and UpdateJMassMatrix on all the rank's cores):
 * the push over contiguous particle ranges; the particles then bucketed by
 * block (counting sort, the re-binning's relinking); the deposit over
 * contiguous block ranges of about equal particle counts, so every cell's
 * blocks are written by one thread, in particle order.  Per-particle results
 * are those of orc_amr_push / orc_amr_deposit; only the order of the energy
 * sum differs.  Returns the kinetic energy.  sel (may be NULL: every block)
 * restricts the deposit to the blocks with sel[b] != 0: the others are
 * neither cleared nor deposited (a bounded sample of the step: the particles of
 * some blocks, pushed, and those blocks' ProcessCell). */
typedef struct {
  const orc_amr* g;
  long p0, p1;
  int b0, b1;
  double* x;
  double* v;
  const uint8_t* spec;
  const double* wcorr;
  int32_t* block;
  int32_t* cell;
  const double *E_half, *Bc_prev, *Bc_cur;
  double *cellJ, *cellM;
  const long* start;   /* per block: first index into order */
  const long* order;   /* particle indices bucketed by block */
  const uint8_t* sel;  /* blocks to deposit, NULL: all */
  double energy;
} mt_task;

static void* mt_push(void* arg) {
  mt_task* t = (mt_task*)arg;
  orc_amr_push(t->g, t->p1 - t->p0, t->x + 3 * t->p0, t->v + 3 * t->p0, t->spec + t->p0,
               t->block + t->p0, t->cell + t->p0, t->E_half, t->Bc_prev);
  return NULL;
}

static void* mt_deposit(void* arg) {
  mt_task* t = (mt_task*)arg;
  double e = 0.0;
  for (int b = t->b0; b < t->b1; b++) {
    if (t->sel && !t->sel[b]) continue;
    memset(t->cellJ + (long)b * 512 * 24, 0, sizeof(double) * 512 * 24);
    memset(t->cellM + (long)b * 512 * 324, 0, sizeof(double) * 512 * 324);
    for (long k = t->start[b]; k < t->start[b + 1]; k++)
      e += deposit_one(t->g, t->order[k], t->x, t->v, t->spec, t->wcorr, t->block, t->cell,
                       t->Bc_cur, t->cellJ, t->cellM);
  }
  t->energy = e;
  return NULL;
}

double orc_amr_push_deposit_mt(const orc_amr* g, long n, double* x, double* v, const uint8_t* spec,
                               const double* wcorr, int32_t* block, int32_t* cell,
                               const double* E_half, const double* Bc_prev, const double* Bc_cur,
                               double* cellJ, double* cellM, int nthreads, const uint8_t* sel) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  mt_task task[256];
  const int nb = g->nblocks;
  for (int t = 0; t < nthreads; t++) {
    mt_task* k = task + t;
    memset(k, 0, sizeof(*k));
    k->g = g; k->x = x; k->v = v; k->spec = spec; k->wcorr = wcorr; k->block = block; k->cell = cell;
    k->E_half = E_half; k->Bc_prev = Bc_prev; k->Bc_cur = Bc_cur; k->cellJ = cellJ; k->cellM = cellM;
    k->p0 = n * t / nthreads;
    k->p1 = n * (t + 1) / nthreads;
  }
  for (int t = 0; t < nthreads; t++) pthread_create(th + t, NULL, mt_push, task + t);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  /* bucket by block (deleted particles, block < 0, are left out) */
  long* start = (long*)calloc((size_t)nb + 1, sizeof(long));
  long* order = (long*)malloc(sizeof(long) * (size_t)(n > 0 ? n : 1));
  for (long p = 0; p < n; p++)
    if (block[p] >= 0) start[block[p] + 1]++;
  for (int b = 0; b < nb; b++) start[b + 1] += start[b];
  long* fill = (long*)malloc(sizeof(long) * (size_t)(nb > 0 ? nb : 1));
  memcpy(fill, start, sizeof(long) * (size_t)nb);
  for (long p = 0; p < n; p++)
    if (block[p] >= 0) order[fill[block[p]]++] = p;
  free(fill);
  /* block ranges of about equal particle counts */
  int b = 0;
  const long tot = start[nb];
  for (int t = 0; t < nthreads; t++) {
    task[t].b0 = b;
    const long target = tot * (t + 1) / nthreads;
    while (b < nb && (t == nthreads - 1 || start[b + 1] <= target)) b++;
    task[t].b1 = (t == nthreads - 1) ? nb : b;
    task[t].start = start;
    task[t].order = order;
    task[t].sel = sel;
  }
  for (int t = 0; t < nthreads; t++) pthread_create(th + t, NULL, mt_deposit, task + t);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  double e = 0.0;
  for (int t = 0; t < nthreads; t++) e += task[t].energy;
  free(start);
  free(order);
  return e;
}

/* Species moments on corners (ProcessCell pic_field_solver_ecsim.cpp:2270-2303,
 * flush :2384-2394) with each cell's own volume, summed on the unique corners
 * of the cell (a hanging corner collects the cells of the fine blocks that
 * have it as a corner): out[corner*10*nspec + 10*spec + q]. */
void orc_amr_species_moments(const orc_amr* g, long n, const double* x, const double* v,
                             const uint8_t* spec, const double* wcorr, const int32_t* block,
                             double* out) {
  const int nq = 10 * g->nspec;
  memset(out, 0, sizeof(double) * (size_t)g->ncorners * nq);
  for (long p = 0; p < n; p++) {
    if (block[p] < 0) continue;
    double w[8];
    int cid[8];
    const int b = block[p];
    stencil(g, b, x + 3 * p, w, cid);
    const double dx = bdx(g, b), V = dx * dx * dx;
    const int s = spec[p];
    const double mass = g->m[s] * g->w[s] * (wcorr ? wcorr[p] : 1.0);
    const double* u = v + 3 * p;
    for (int c = 0; c < 8; c++) {
      const double t = mass * w[c], t0 = t * u[0], t1 = t * u[1], t2 = t * u[2];
      double* o = out + (size_t)cid[c] * nq + 10 * s;
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

/* curl of the cell from its 8 corner values (table order): C x */
static void cell_curl(const double e[8][3], double dx, double out[3]) {
  double dEz_dy = 0, dEy_dz = 0, dEx_dz = 0, dEz_dx = 0, dEy_dx = 0, dEx_dy = 0;
  for (int c = 0; c < 8; c++) {
    const double sx = kOff[c][0] ? 1.0 : -1.0, sy = kOff[c][1] ? 1.0 : -1.0,
                 sz = kOff[c][2] ? 1.0 : -1.0;
    dEz_dy += sy * e[c][2]; dEy_dz += sz * e[c][1];
    dEx_dz += sz * e[c][0]; dEz_dx += sx * e[c][2];
    dEy_dx += sx * e[c][1]; dEx_dy += sy * e[c][0];
  }
  const double f = 0.25 / dx;
  out[0] = f * (dEz_dy - dEy_dz);
  out[1] = f * (dEx_dz - dEz_dx);
  out[2] = f * (dEy_dx - dEx_dy);
}

/* C^T y scattered onto the 8 corners (adds s * C^T y) */
static void cell_curl_t(const double y[3], double dx, double s, double out[8][3]) {
  const double f = 0.25 / dx * s;
  for (int c = 0; c < 8; c++) {
    const double sx = kOff[c][0] ? 1.0 : -1.0, sy = kOff[c][1] ? 1.0 : -1.0,
                 sz = kOff[c][2] ? 1.0 : -1.0;
    out[c][0] += f * (sz * y[1] - sy * y[2]);
    out[c][1] += f * (sx * y[2] - sz * y[0]);
    out[c][2] += f * (sy * y[0] - sx * y[1]);
  }
}

static int pair_index(int a, int b) {
  const int hi = a > b ? a : b, lo = a > b ? b : a;
  return hi * (hi + 1) / 2 + lo;
}

/* y = A x on the full corner vector (free rows: P^T A P x; hanging rows: x_h - (P x)_h).
 * with_identity/with_curl/with_mass select the operator pieces (all on for the solve). */
void orc_amr_apply(const orc_amr* g, const double* cellM, const double* x, double* y,
                   int with_identity, int with_curl, int with_mass) {
  const int nc = g->ncorners;
  memset(y, 0, sizeof(double) * 3 * nc);
  const double f = 4.0 * PI_D * g->dt * g->theta, th2 = g->theta * g->theta * g->dt * g->dt;
  for (int b = 0; b < g->nblocks; b++) {
    const double dx = bdx(g, b), V = dx * dx * dx;
    for (int l = 0; l < 512; l++) {
      const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
      int cid[8];
      double e[8][3], out[8][3];
      memset(out, 0, sizeof(out));
      for (int c = 0; c < 8; c++) {
        cid[c] = cell_corner(g, b, i + kOff[c][0], j + kOff[c][1], k + kOff[c][2]);
        corner_val(g, x, cid[c], e[c]);
      }
      if (with_identity)
        for (int c = 0; c < 8; c++)
          for (int d = 0; d < 3; d++) out[c][d] += 0.125 * V * e[c][d];
      if (with_curl) {
        double cu[3];
        cell_curl(e, dx, cu);
        cell_curl_t(cu, dx, th2 * V, out);
      }
      if (with_mass) {
        const double* mm = cellM + ((long)b * 512 + l) * 324;
        for (int a = 0; a < 8; a++)
          for (int c2 = 0; c2 < 8; c2++) {
            const double* blk = mm + pair_index(a, c2) * 9;
            for (int p = 0; p < 3; p++)
              for (int q = 0; q < 3; q++) out[a][p] += f * V * blk[3 * p + q] * e[c2][q];
          }
      }
      /* scatter with P^T */
      for (int c = 0; c < 8; c++) {
        const int cc = cid[c], s = g->hang_start[cc], en = g->hang_start[cc + 1];
        if (s == en) {
          for (int d = 0; d < 3; d++) y[3 * cc + d] += out[c][d];
        } else {
          for (int t = s; t < en; t++)
            for (int d = 0; d < 3; d++) y[3 * g->hang_parent[t] + d] += g->hang_weight[t] * out[c][d];
        }
      }
    }
  }
  /* hanging rows: constraint */
  for (int c = 0; c < nc; c++) {
    const int s = g->hang_start[c], en = g->hang_start[c + 1];
    if (s == en) continue;
    double pv[3];
    corner_val(g, x, c, pv);
    for (int d = 0; d < 3; d++) y[3 * c + d] = x[3 * c + d] - pv[d];
  }
  /* boundary rows of open axes (GetStencil's boundary_short_circuit,
   * get_stencil.cpp:440-620): Dirichlet dE_b = 0, Neumann dE_b = mean of the
   * inward face-normal donors */
  if (g->bnd_flag)
    for (int c = 0; c < nc; c++) {
      if (!g->bnd_flag[c]) continue;
      for (int d = 0; d < 3; d++) {
        double v = x[3 * c + d];
        for (int t = g->bnd_start[c]; t < g->bnd_start[c + 1]; t++)
          v -= g->bnd_weight[t] * x[3 * g->bnd_col[t] + d];
        y[3 * c + d] = v;
      }
    }
}

/* RHS in weak form: sum_cells V [theta c dt C^T B - (theta c dt)^2 C^T C E^n - f M E^n] - f J_weak,
 * with J_weak = sum_cells cellJ (no 1/V); hanging rows 0. */
void orc_amr_rhs(const orc_amr* g, const double* E_n, const double* Bcen, const double* cellJ,
                 const double* cellM, double* rhs) {
  const int nc = g->ncorners;
  double* tmp = (double*)malloc(sizeof(double) * 3 * nc);
  orc_amr_apply(g, cellM, E_n, tmp, 0, 1, 1);
  const double f = 4.0 * PI_D * g->dt * g->theta;
  for (long i = 0; i < 3L * nc; i++) rhs[i] = -tmp[i];
  for (int b = 0; b < g->nblocks; b++) {
    const double dx = bdx(g, b), V = dx * dx * dx;
    for (int l = 0; l < 512; l++) {
      const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
      const long cl = (long)b * 512 + l;
      double out[8][3];
      memset(out, 0, sizeof(out));
      cell_curl_t(Bcen + 3 * cl, dx, g->theta * g->dt * V, out);
      for (int c = 0; c < 8; c++)
        for (int d = 0; d < 3; d++) out[c][d] -= f * cellJ[cl * 24 + 3 * c + d];
      for (int c = 0; c < 8; c++) {
        const int cc = cell_corner(g, b, i + kOff[c][0], j + kOff[c][1], k + kOff[c][2]);
        const int s = g->hang_start[cc], en = g->hang_start[cc + 1];
        if (s == en) {
          for (int d = 0; d < 3; d++) rhs[3 * cc + d] += out[c][d];
        } else {
          for (int t = s; t < en; t++)
            for (int d = 0; d < 3; d++) rhs[3 * g->hang_parent[t] + d] += g->hang_weight[t] * out[c][d];
        }
      }
    }
  }
  for (int c = 0; c < nc; c++)
    if (g->hang_start[c + 1] > g->hang_start[c] || (g->bnd_flag && g->bnd_flag[c]))
      for (int d = 0; d < 3; d++) rhs[3 * c + d] = 0.0;
  free(tmp);
}

static double dotv(long n, const double* a, const double* b) {
  double s = 0.0;
  for (long i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* restarted GMRES(m), x0 = 0, no preconditioner; stop on ||b-Ax|| <= tol ||b|| */
int orc_amr_gmres(const orc_amr* g, const double* cellM, const double* b, double* x, double tol,
                  int maxit, int restart, double* resid_out) {
  const long n = 3L * g->ncorners;
  const int m = restart;
  double* V = (double*)malloc(sizeof(double) * n * (m + 1));
  double* w = (double*)malloc(sizeof(double) * n);
  double* H = (double*)calloc((size_t)(m + 1) * m, sizeof(double));
  double *cs = (double*)malloc(sizeof(double) * m), *sn = (double*)malloc(sizeof(double) * m);
  double* s = (double*)malloc(sizeof(double) * (m + 1));
  double* yv = (double*)malloc(sizeof(double) * m);
  for (long i = 0; i < n; i++) x[i] = 0.0;
  const double bn = sqrt(dotv(n, b, b));
  int it = 0, conv = 0;
  double rel = 0.0;
  if (bn == 0.0) { conv = 1; goto done; }
  while (it < maxit) {
    orc_amr_apply(g, cellM, x, w, 1, 1, 1);
    for (long i = 0; i < n; i++) V[i] = b[i] - w[i];
    double beta = sqrt(dotv(n, V, V));
    rel = beta / bn;
    if (rel <= tol) { conv = 1; break; }
    for (long i = 0; i < n; i++) V[i] /= beta;
    for (int i = 0; i <= m; i++) s[i] = 0.0;
    s[0] = beta;
    int j;
    for (j = 0; j < m && it < maxit; j++) {
      it++;
      orc_amr_apply(g, cellM, V + (long)j * n, w, 1, 1, 1);
      for (int i = 0; i <= j; i++) {
        double hh = dotv(n, w, V + (long)i * n);
        H[i * m + j] = hh;
        for (long t = 0; t < n; t++) w[t] -= hh * V[(long)i * n + t];
      }
      double hn = sqrt(dotv(n, w, w));
      H[(j + 1) * m + j] = hn;
      for (long t = 0; t < n; t++) V[(long)(j + 1) * n + t] = hn > 0 ? w[t] / hn : 0.0;
      for (int i = 0; i < j; i++) {
        double a = H[i * m + j], c = H[(i + 1) * m + j];
        H[i * m + j] = cs[i] * a + sn[i] * c;
        H[(i + 1) * m + j] = -sn[i] * a + cs[i] * c;
      }
      double a = H[j * m + j], c = H[(j + 1) * m + j], r = sqrt(a * a + c * c);
      cs[j] = r > 0 ? a / r : 1.0;
      sn[j] = r > 0 ? c / r : 0.0;
      H[j * m + j] = r;
      H[(j + 1) * m + j] = 0.0;
      s[j + 1] = -sn[j] * s[j];
      s[j] = cs[j] * s[j];
      rel = fabs(s[j + 1]) / bn;
      if (rel <= tol) { j++; break; }
    }
    for (int i = j - 1; i >= 0; i--) {
      double t = s[i];
      for (int k = i + 1; k < j; k++) t -= H[i * m + k] * yv[k];
      yv[i] = t / H[i * m + i];
    }
    for (long t = 0; t < n; t++) {
      double acc = 0.0;
      for (int i = 0; i < j; i++) acc += yv[i] * V[(long)i * n + t];
      x[t] += acc;
    }
    if (rel <= tol) {
      orc_amr_apply(g, cellM, x, w, 1, 1, 1);
      for (long i = 0; i < n; i++) w[i] = b[i] - w[i];
      rel = sqrt(dotv(n, w, w)) / bn;
      if (rel <= 10 * tol) { conv = 1; break; }
    }
  }
done:
  if (resid_out) *resid_out = rel;
  free(V); free(w); free(H); free(cs); free(sn); free(s); free(yv);
  return conv ? it : -it;
}

/* B^{n+1} = B^n - c dt C E^{n+theta} per cell */
void orc_amr_update_b(const orc_amr* g, const double* E_half, const double* Bn, double* Bnp1) {
  for (int b = 0; b < g->nblocks; b++) {
    const double dx = bdx(g, b);
    for (int l = 0; l < 512; l++) {
      const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
      double e[8][3], cu[3];
      for (int c = 0; c < 8; c++)
        corner_val(g, E_half, cell_corner(g, b, i + kOff[c][0], j + kOff[c][1], k + kOff[c][2]), e[c]);
      cell_curl(e, dx, cu);
      const long cl = (long)b * 512 + l;
      for (int d = 0; d < 3; d++) Bnp1[3 * cl + d] = Bn[3 * cl + d] - g->dt * cu[d];
    }
  }
  if (!g->open_mask) return;
  /* UpdateB's boundary branch (pic_field_solver_ecsim.cpp:5274-5600) on the
   * cells with a face on an open domain face: Dirichlet keeps B^n; Neumann
   * takes the mean of B^{n+1} of the face-normal inward neighbours (one per
   * such face, same block), faces before edges before corners; a cell on any
   * Neumann face is Neumann (domain_bc.cpp:49-63 marks those faces last) */
  for (int pass = 0; pass <= (g->field_bc ? 3 : 0); pass++)
    for (int b = 0; b < g->nblocks; b++) {
      const int st = 1 << (g->lmax - g->level[b]);
      for (int l = 0; l < 512; l++) {
        const int idx[3] = {l & 7, (l >> 3) & 7, l >> 6};
        int side[3] = {0, 0, 0}, nface = 0;
        for (int d = 0; d < 3; d++) {
          if (!((g->open_mask >> d) & 1)) continue;
          const int lo = g->origin[3 * b + d] + idx[d] * st;
          if (lo == 0) side[d] = -1;
          else if (lo + st == g->nfine[d]) side[d] = 1;
          nface += side[d] != 0;
        }
        if (!nface) continue;
        const long cl = (long)b * 512 + l;
        int neu = 0;
        for (int d = 0; d < 3; d++)
          if (side[d]) neu |= (g->field_bc >> (2 * d + (side[d] > 0))) & 1;
        if (!neu) {
          if (pass == 0)
            for (int q = 0; q < 3; q++) Bnp1[3 * cl + q] = Bn[3 * cl + q];
          continue;
        }
        if (nface != pass) continue;
        double acc[3] = {0.0, 0.0, 0.0};
        for (int d = 0; d < 3; d++) {
          if (!side[d]) continue;
          int j[3] = {idx[0], idx[1], idx[2]};
          j[d] -= side[d];
          const long dn = (long)b * 512 + j[0] + 8 * (j[1] + 8 * j[2]);
          for (int q = 0; q < 3; q++) acc[q] += Bnp1[3 * dn + q];
        }
        for (int q = 0; q < 3; q++) Bnp1[3 * cl + q] = acc[q] / nface;
      }
    }
}

/* corner B: volume-weighted mean of the touching cells; hanging corners interpolated */
void orc_amr_c2n(const orc_amr* g, const double* Bcen, double* Bcor) {
  const int nc = g->ncorners;
  double* wsum = (double*)calloc((size_t)nc, sizeof(double));
  memset(Bcor, 0, sizeof(double) * 3 * nc);
  for (int b = 0; b < g->nblocks; b++) {
    const double dx = bdx(g, b), V = dx * dx * dx;
    for (int l = 0; l < 512; l++) {
      const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
      const long cl = (long)b * 512 + l;
      for (int c = 0; c < 8; c++) {
        const int cc = cell_corner(g, b, i + kOff[c][0], j + kOff[c][1], k + kOff[c][2]);
        wsum[cc] += V;
        for (int d = 0; d < 3; d++) Bcor[3 * cc + d] += V * Bcen[3 * cl + d];
      }
    }
  }
  for (int c = 0; c < nc; c++)
    if (wsum[c] > 0)
      for (int d = 0; d < 3; d++) Bcor[3 * c + d] /= wsum[c];
  for (int c = 0; c < nc; c++) {
    if (g->hang_start[c + 1] == g->hang_start[c]) continue;
    double v[3];
    corner_val(g, Bcor, c, v);
    for (int d = 0; d < 3; d++) Bcor[3 * c + d] = v[d];
  }
  free(wsum);
}

/* E^{n+1} in place; hanging corners re-interpolated.  Returns the wave energy
 * sum_cells V (sum_corners |E|^2 / 8 + |B|^2) / (8 pi). */
double orc_amr_update_e(const orc_amr* g, const double* E_half, double* E_n, const double* Bcen) {
  const int nc = g->ncorners;
  const double th = g->theta;
  for (long i = 0; i < 3L * nc; i++) E_n[i] = (E_half[i] - (1.0 - th) * E_n[i]) / th;
  for (int c = 0; c < nc; c++) {
    if (g->hang_start[c + 1] == g->hang_start[c]) continue;
    double v[3];
    corner_val(g, E_n, c, v);
    for (int d = 0; d < 3; d++) E_n[3 * c + d] = v[d];
  }
  double sum = 0.0;
  for (int b = 0; b < g->nblocks; b++) {
    const double dx = bdx(g, b), V = dx * dx * dx;
    for (int l = 0; l < 512; l++) {
      const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
      const long cl = (long)b * 512 + l;
      double e2 = 0.0;
      for (int c = 0; c < 8; c++) {
        double v[3];
        corner_val(g, E_n, cell_corner(g, b, i + kOff[c][0], j + kOff[c][1], k + kOff[c][2]), v);
        e2 += v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
      }
      const double* B = Bcen + 3 * cl;
      sum += (0.125 * e2 + B[0] * B[0] + B[1] * B[1] + B[2] * B[2]) * V * 0.125 / PI_D;
    }
  }
  return sum;
}

/* one ECSIM step on the AMR mesh (reference order of pic_time_step.cpp:403-551) */
int orc_amr_step(const orc_amr* g, long n, double* x, double* v, const uint8_t* spec,
                 const double* wcorr, int32_t* block, int32_t* cell, double* E_n, double* E_half,
                 double* Bcen, double* Bcor_prev, double* Bcor_cur, double* cellJ, double* cellM,
                 double tol, int maxit, double* diag) {
  const int nc = g->ncorners;
  const long ncell = (long)g->nblocks * 512;
  double* rhs = (double*)malloc(sizeof(double) * 3 * nc);
  double* dE = (double*)malloc(sizeof(double) * 3 * nc);
  double* Bnew = (double*)malloc(sizeof(double) * 3 * ncell);
  double resid = 0.0;
  orc_amr_rhs(g, E_n, Bcen, cellJ, cellM, rhs);
  int it = orc_amr_gmres(g, cellM, rhs, dE, tol, maxit, 30, &resid);
  for (long i = 0; i < 3L * nc; i++) E_half[i] = E_n[i] + dE[i];
  orc_amr_update_b(g, E_half, Bcen, Bnew);
  memcpy(Bcen, Bnew, sizeof(double) * 3 * ncell);
  memcpy(Bcor_prev, Bcor_cur, sizeof(double) * 3 * nc);
  orc_amr_c2n(g, Bcen, Bcor_cur);
  double wave = orc_amr_update_e(g, E_half, E_n, Bcen);
  orc_amr_push(g, n, x, v, spec, block, cell, E_half, Bcor_prev);
  double pe = orc_amr_deposit(g, n, x, v, spec, wcorr, block, cell, Bcor_cur, cellJ, cellM);
  if (diag) { diag[0] = pe; diag[1] = wave; diag[2] = resid; }
  free(rhs); free(dE); free(Bnew);
  return it;
}
