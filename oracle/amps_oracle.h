/*
 * amps_oracle.h -- FP64 CPU restatement of the AMPS particle / ECSIM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code: it is the checker that tests/, __graft_entry__.smoke() and
 * the cpu_baseline leg of bench.py compare the CUDA path against.
 *
 * Scope: a periodic box of nbx*nby*nbz uniform blocks of 8^3 cells, two or
 * more species, corner-based E and B (the _PIC_FIELD_SOLVER_B_CORNER_BASED_
 * configuration), normalised units (c = E_conv = B_conv = length_conv = 1).
 * Every function cites the reference file:line it restates.
 *
 * Parity: the 81-point operator coefficients are pinned against the
 * reference's own stencil library (src/general/stencil.h) through
 * oracle/pins/stencil_pin.cpp.  ProcessCell (J, M, particle energy, cflCell),
 * Lapenta2017 and Boris are pinned against the reference's own
 * pic_field_solver_ecsim.cpp, pic_mover_boris.cpp and
 * pic_interpolation_routines.cpp, compiled with a hand-written configuration
 * by oracle/pins/ecsim_pin.cpp (golden tests/golden/ecsim_ref.json; equal to
 * 1e-13, bit-identical on x86).  The field update is pinned by the
 * conservation law ECSIM is built on (theta = 0.5 conserves total energy to
 * the linear-solver tolerance).
 * The GMRES is absent from the reference (SWMF share/Library), so its
 * parity is unpinned: the stop rule is stated explicitly instead.
 */
#ifndef AMPS_ORACLE_H
#define AMPS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NC 8              /* cells per block edge (_BLOCK_CELLS_X_) */
#define ORC_MAXSPEC 8

typedef struct {
  int nbx, nby, nbz;          /* blocks per axis */
  double x0[3];               /* domain origin */
  double dx[3];               /* cell size */
  int nspec;
  double q[ORC_MAXSPEC];      /* normalised charge per species */
  double m[ORC_MAXSPEC];      /* normalised mass per species */
  double w[ORC_MAXSPEC];      /* macro-particle weight per species */
  double dt, theta;
} orc_mesh;

/* ---- stencil coefficient tables (27 taps, index ii+3jj+9kk with offsets
 *      {0,-1,+1} for ii,jj,kk = 0,1,2 as in the reference's indexAddition) */
void orc_laplacian_table(int axis, double out[27]);
void orc_graddiv_table(int p, int q, double out[27]);

/* ---- interpolation / push / deposition ---- */
/* 1: the B arguments of orc_push / orc_deposit (and the ECSIM step's) are cell
 * arrays interpolated from the cell centres (_PIC_FIELD_SOLVER_B_CENTER_BASED_);
 * 0 (default): corner arrays */
void orc_set_b_center(int on);
/* B at n located points from a cell-centred field (the centre-B stencil) */
void orc_centre_b_at(const orc_mesh* g, long n, const double* x, const int32_t* block,
                     const double* Bc, double* B);
void orc_corner_weights(const double xloc[3], double w_table[8]);
long orc_push(const orc_mesh* g, long n, double* x, double* v, const uint8_t* spec,
              int32_t* block, int32_t* cell, const double* E_half, const double* Bc_prev);
/* Mover::Relativistic::Boris on the mesh corner fields E, B (sub-stepped by the
 * gyro period); returns the number of sub-steps */
long orc_relboris(const orc_mesh* g, long n, double* x, double* v, const uint8_t* spec,
                  int32_t* block, int32_t* cell, const double* E, const double* B, double dt_total,
                  double c_light);
double orc_deposit(const orc_mesh* g, long n, const double* x, const double* v,
                   const uint8_t* spec, const double* wcorr, const int32_t* block,
                   const int32_t* cell, const double* Bc_cur, double* J, double* M);
void orc_locate(const orc_mesh* g, long n, const double* x, int32_t* block, int32_t* cell);
long orc_boris(const orc_mesh* g, long n, double* x, double* v, const uint8_t* spec,
               int32_t* block, int32_t* cell, const double* E, const double* B, double dt);
void orc_cfl(const orc_mesh* g, long n, const double* v, const uint8_t* spec,
             const int32_t* block, const int32_t* cell, double* cfl_max);

/* Mover::Boris (src/pic/pic_mover_boris.cpp:126-553, scalar path :264-290)
 * with the Lorentz force of BorisSplitAcceleration_default (:104-112):
 * accl = (q/m) E, rotation = -(q/m) B, u = v + dt/2 accl, h = -dt/2 rotation,
 * U = ((1-h^2) u + 2 (u x h + (u.h) h)) / (1+h^2), v' = U + dt/2 accl. */
static inline void orc_boris_velocity(double qm, double dt, const double E[3], const double B[3],
                                      double v[3]) {
  double accl[3], rot[3], u[3], h[3], U[3];
  const double dt2 = dt / 2.0;
  for (int d = 0; d < 3; d++) {
    accl[d] = 0.0 + qm * E[d];
    rot[d] = 0.0 - qm * B[d];
  }
  for (int d = 0; d < 3; d++) {
    u[d] = v[d] + dt2 * accl[d];
    h[d] = -dt2 * rot[d];
  }
  const double h2 = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
  const double uh = u[0] * h[0] + u[1] * h[1] + u[2] * h[2];
  U[0] = ((1 - h2) * u[0] + 2 * (u[1] * h[2] - h[1] * u[2] + uh * h[0])) / (1 + h2);
  U[1] = ((1 - h2) * u[1] + 2 * (u[2] * h[0] - h[2] * u[0] + uh * h[1])) / (1 + h2);
  U[2] = ((1 - h2) * u[2] + 2 * (u[0] * h[1] - h[0] * u[1] + uh * h[2])) / (1 + h2);
  for (int d = 0; d < 3; d++) v[d] = U[d] + dt2 * accl[d];
}

/* ---- field solve ---- */
void orc_center_to_corner(const orc_mesh* g, const double* Bcen, double* Bcor);
/* open axes (bit d): particles leaving the domain through their faces are
 * deleted by the pushes (block = cell = -1), on uniform and AMR meshes */
void orc_set_open_axes(int mask);
/* OpenFlow injection through one face (see amps_oracle.c): up to cap new
 * particles; returns the number kept, -1 if the velocity sampling ran out */
long orc_inject(const orc_mesh* g, int face, int spec, double density, const double drift[3],
                double vth, unsigned long long seed, unsigned long long step, int src,
                const double* E_half, const double* Bc_prev, long cap, double* xo, double* vo,
                int32_t* blk, int32_t* cel);
/* species moments on corners (ProcessCell :2270-2303): out[corner][10*nspec] */
void orc_species_moments(const orc_mesh* g, long n, const double* x, const double* v,
                         const uint8_t* spec, const double* wcorr, const int32_t* block,
                         const int32_t* cell, double* out);
void orc_rhs(const orc_mesh* g, const double* E_n, const double* Bcen, const double* J,
             const double* M, double* rhs);
void orc_matvec(const orc_mesh* g, const double* M, const double* x, double* y);
void orc_jacobi_diag(const orc_mesh* g, const double* M, double* diag);
int orc_gmres(const orc_mesh* g, const double* M, const double* b, double* x, double tol,
              int maxit, int restart, int precond, double* resid_out);
void orc_update_b(const orc_mesh* g, const double* E_half, const double* B_n, double* B_np1);
double orc_update_e(const orc_mesh* g, const double* E_half, double* E_n, const double* B_cen);

/* ---- one full ECSIM time step in the reference order (pic_time_step.cpp:403-551) ----
 * state arrays: E_n, E_half, Bcen (B^n on entry, B^{n+1} on exit), Bcor_prev/
 * Bcor_cur (corner B, swapped), J, M (deposited at the end of the previous step).
 * Returns GMRES iterations; energies are written to diag[0..2] =
 * {particle energy, wave energy, gmres relative residual}. */
int orc_ecsim_step(const orc_mesh* g, long n, double* x, double* v, const uint8_t* spec,
                   const double* wcorr, int32_t* block, int32_t* cell, double* E_n,
                   double* E_half, double* Bcen, double* Bcor_prev, double* Bcor_cur,
                   double* J, double* M, double tol, int maxit, int precond, double* diag);

/* ---- restart particle section and checksum (src/pic/pic_restart.cpp) ----
 * The CRC32 class of src/general/specfunc.h:438-505 in its 64-bit accumulator
 * (the reference's `unsigned long`).  The class cannot be compiled from the
 * reference here (specfunc.h needs MPI), so its low half is pinned by the
 * published check value of the MSB-first 0x04C11DB7 CRC with initial value 0
 * (CRC-32/POSIX before its final xor) and the high half by the recurrence. */
void orc_crc32_table(uint64_t t[256]);
uint64_t orc_crc32_add(uint64_t acc, const uint8_t* p, long n);

typedef struct {
  int len, off_v, off_x, off_sp, off_w;   /* off_w < 0: no weight correction */
} orc_record_layout;

/* Particles in any order in which each (block, cell) keeps its list order;
 * cell = i + 8 (j + 8 k).  blocks in block_order (NULL: 0..nb-1).  Returns the
 * section's size (bytes written when out != NULL, -1 when cap is too small). */
long long orc_restart_pack(const orc_record_layout* L, int nb, const int32_t* block_order,
                           const uint8_t* node_ids, int id_len, int nspec, const double* weight,
                           long n, const double* x, const double* v, const uint8_t* spec,
                           const double* wcorr, const int32_t* block, const int32_t* cell,
                           uint8_t* out, long long cap);
/* GetParticleDataCheckSum over the same particles (links zeroed) */
uint64_t orc_particle_checksum(const orc_record_layout* L, int nb, const int32_t* block_order, long n,
                               const double* x, const double* v, const uint8_t* spec,
                               const double* wcorr, const int32_t* block, const int32_t* cell);

/* ---- div E correction on the periodic uniform mesh (amps_oracle_dive.c;
 *      ECSIM::divECorrection, pic_field_solver_ecsim.cpp:4341-4364) ---- */
void orc_net_charge(const orc_mesh* g, long n, const double* x, const uint8_t* spec,
                    const double* wcorr, const int32_t* block, double* rho);
void orc_div_e(const orc_mesh* g, const double* E, double* dive);
void orc_poisson_rhs(const orc_mesh* g, const double* rho_new, const double* rho_old,
                     const double* dive, double* rhs);
int orc_poisson_cg(const orc_mesh* g, const double* rhs, double* phi, double tol, int maxit,
                   double* rel);
void orc_corner_charge(const orc_mesh* g, long n, const double* x, const uint8_t* spec,
                       const double* wcorr, const int32_t* block, const int32_t* cell, int s0,
                       double* cq);
long orc_dive_correct(const orc_mesh* g, long n, double* x, const uint8_t* spec,
                      const int32_t* block, const int32_t* cell, const double* phi,
                      const double* cq);
void orc_div_e_correction(const orc_mesh* g, long n, double* x, const uint8_t* spec,
                          const double* wcorr, int32_t* block, int32_t* cell, const double* E,
                          double* rho_new, double* rho_old, double* dive, double* phi, int first,
                          double tol, int maxit, double* stats);

/* ---- relativistic Boris, gridless form (srcEarth/gridless/GridlessParticleMovers.cpp:781) ---- */
void orc_dipole_b(const double x[3], double b_eq, double r_e, const double b_ext[3], double B[3]);
long orc_trace(long n, double* x, double* p, int32_t* status, int64_t* steps, double q, double m0,
               double b_eq, double r_e, const double b_ext[3], double r_in, double r_out,
               long max_steps, double dphi_max, double dt_max, int single_precision);

#ifdef __cplusplus
}
#endif
#endif
