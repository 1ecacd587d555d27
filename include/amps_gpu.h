/*
 * amps_gpu.h -- C ABI of libamps_gpu.so, the GB300 (sm_103a) implementation of
 * the AMPS particle / ECSIM hot path.
 *
 * The entry points mirror the reference call surfaces they replace:
 *   PIC::Mover::MoveParticles           src/pic/pic_mover.cpp:580
 *   PIC::Mover::Lapenta2017             src/pic/pic_mover_boris.cpp:837-1380
 *   ECSIM::UpdateJMassMatrix            src/pic/pic_field_solver_ecsim.cpp:3244
 *   ECSIM::TimeStep                     src/pic/pic_field_solver_ecsim.cpp:6179
 *   cLinearSystemCornerNode::Solve      srcInterface/LinearSystemCornerNode.h:3212
 *   PIC::ParticleBuffer (import/export) src/pic/pic.h:2716-3846
 *   gridless BorisStep tracing          srcEarth/gridless/GridlessParticleMovers.cpp:781
 *
 * Conventions
 *   - Plain pointers to HOST memory unless a name says otherwise; sizes are
 *     element counts.  No call aborts: every call returns amps_gpu_status and
 *     amps_gpu_last_error() describes the last failure of a context.
 *   - Units are the reference's normalised ECSIM units
 *     (_PIC_FIELD_SOLVER_INPUT_UNIT_NORM_: c = E_conv = B_conv = 1); charge
 *     and mass tables are passed already normalised (picunits::si2no_q/_m).
 *   - Field arrays on the host side use the global periodic corner numbering
 *     idx(I,J,K) = I + NX*(J + NY*K) with NX = 8*nbx, three interleaved
 *     components per node (x,y,z); the mass matrix is 243 values per corner:
 *     27 neighbour slots x row-major 3x3, slot = ii + 3*jj + 9*kk where
 *     ii,jj,kk = 0,1,2 stand for offsets 0,-1,+1 (the reference's
 *     MassMatrixOffsetTable, pic_field_solver_ecsim.cpp:624-640).
 *   - Particle block ids are bx + nbx*(by + nby*bz); cell ids are block-local
 *     i + 8*(j + 8*k) (the reference's _getCenterNodeLocalNumber order).
 *   - A context owns one CUDA stream; it is not thread safe.
 */
#ifndef AMPS_GPU_H
#define AMPS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AMPS_GPU_MAX_SPECIES 8

/* Replaces the reference's exit(__LINE__,__FILE__,msg) aborts
 * (src/general/global.h:50) and the mover return codes (src/pic/pic.h:5955-5960). */
typedef enum {
  AMPS_GPU_OK = 0,
  AMPS_GPU_INVALID_ARG = 1,
  AMPS_GPU_OUT_OF_DOMAIN_PARTICLES = 2,
  AMPS_GPU_GMRES_NOT_CONVERGED = 3,
  AMPS_GPU_DEVICE_TIMEOUT = 4,
  AMPS_GPU_CUDA_ERROR = 5,
  AMPS_GPU_CAPACITY_EXCEEDED = 6,
  AMPS_GPU_NO_DEVICE = 7
} amps_gpu_status;

typedef struct amps_gpu_ctx amps_gpu_ctx;

/* Mesh, species and time-step parameters.  The mesh is a periodic box of
 * nbx*nby*nbz uniform blocks of 8^3 cells (_BLOCK_CELLS_X_ = 8), which is the
 * domain + ghost-block layout of Periodic::ExchangeParticles
 * (src/pic/pic_bc_periodic.cpp:55) with the ghost layer folded away. */
typedef struct {
  int nbx, nby, nbz;
  double x0[3];                 /* domain origin (xGlobalMin) */
  double dx[3];                 /* cell size */
  int nspec;
  double charge[AMPS_GPU_MAX_SPECIES]; /* normalised charge (ElectricChargeTable) */
  double mass[AMPS_GPU_MAX_SPECIES];   /* normalised mass (MolMass) */
  double weight[AMPS_GPU_MAX_SPECIES]; /* macro-particle weight (GetLocalParticleWeight) */
  double dt;                    /* GlobalTimeStep[0] */
  double theta;                 /* ECSIM::theta (0.5) */
  long long particle_capacity;  /* maximum particles held on the device */
  int track_ids;                /* 1: carry a 32-bit particle id through re-binning */
  int device;                   /* CUDA device ordinal */
} amps_gpu_config;

typedef struct {
  int iterations;               /* GMRES iterations (matrix-vector products after the first) */
  int converged;
  double rel_residual;          /* ||b - A x|| / ||b|| (true residual at exit) */
  double wave_energy;           /* UpdateE energy sum, pic_field_solver_ecsim.cpp:5995 */
} amps_gpu_solve_stats;

typedef struct {
  amps_gpu_solve_stats solve;
  double particle_energy;       /* UpdateJMassMatrix energy sum, :3972-3987 */
  long long out_of_block;       /* particles that moved more than one block (reported, kept) */
  long long ulp_face;           /* particles that ended within 1 FP32 ulp of a cell face */
} amps_gpu_step_stats;

/* ---- block-structured AMR meshes (leaf blocks of the reference octree,
 *      src/meshAMR/meshAMRgeneric.h) ----
 * A leaf block has 8^3 cells, a refinement level (cell size dx0 / 2^level) and
 * its origin on the finest lattice in finest-cell units.  amps_amr_build checks
 * coverage, non-overlap and 2:1 balance (faces, edges, vertices), numbers the
 * unique corners, and derives the hanging-corner constraints (interpolation
 * from the coarser block's corners) that the reference's same-level stencils
 * (src/pic/ecsim/get_stencil.cpp:1100-1160) leave undefined. */
typedef struct {
  int level;
  int ix, iy, iz;  /* origin, finest-cell units */
} amps_block_desc;

typedef struct amps_amr_mesh amps_amr_mesh;

amps_gpu_status amps_amr_build(int nbx0, int nby0, int nbz0, int lmax, const double* x0,
                               double dx0, const amps_block_desc* blocks, int nblocks,
                               amps_amr_mesh** out);
amps_gpu_status amps_amr_info(const amps_amr_mesh* m, int* nblocks, int* ncorners, int* nhanging,
                              int* nparents, int* nfine);
/* corner_tab[nblocks*729] (block-local corner i+9(j+9k) -> unique corner),
 * corner_xyz[3*ncorners], hang_start[ncorners+1], hang_parent[nparents],
 * hang_weight[nparents], fine_map[finest blocks]; any pointer may be NULL */
amps_gpu_status amps_amr_tables(const amps_amr_mesh* m, int32_t* corner_tab, int32_t* corner_xyz,
                                int32_t* hang_start, int32_t* hang_parent, double* hang_weight,
                                int32_t* fine_map);
amps_gpu_status amps_amr_destroy(amps_amr_mesh* m);
/* A mesh with non-periodic axes (open_axes[d] != 0; the reference's
 * _PIC_BC__PERIODIC_MODE_OFF_ with the field boundary policy of
 * src/pic/ecsim/domain_bc.cpp applied to every domain face): corners keep
 * their positions 0..nfine on open axes, and the free corners on those
 * domain faces become constraint rows of the field solve (GetStencil's
 * boundary_short_circuit, src/pic/ecsim/get_stencil.cpp:440-620):
 * field_bc 0 Dirichlet (dE = 0, the corner keeps E^n), 1 Neumann (dE equals
 * the mean of the inward face-normal donor corners).  The cells on those
 * faces take UpdateB's boundary branch (pic_field_solver_ecsim.cpp:
 * 5274-5600): Dirichlet B^{n+1} = B^n, Neumann B^{n+1} = mean of the inward
 * face-normal donor cells, faces before edges before corners.  Particles
 * leaving through those faces are deleted (amps_gpu_set_open_axes is implied
 * by the mesh). */
amps_gpu_status amps_amr_build_open(int nbx0, int nby0, int nbz0, int lmax, const double* x0,
                                    double dx0, const amps_block_desc* blocks, int nblocks,
                                    const int* open_axes, int field_bc, amps_amr_mesh** out);
/* The same with one field boundary type per domain face (cDomainBC's per-face
 * policy, src/pic/ecsim/domain_bc.cpp:39-45): face_bc[2 d + high] (faces -x,
 * +x, -y, +y, -z, +z), 0 Dirichlet or 1 Neumann; faces of periodic axes are
 * ignored.  A corner or cell on faces of both types is Neumann, its donors
 * along every open face it touches (RecomputeBCType marks the Neumann faces
 * after the Dirichlet ones). */
amps_gpu_status amps_amr_build_open_faces(int nbx0, int nby0, int nbz0, int lmax, const double* x0,
                                          double dx0, const amps_block_desc* blocks, int nblocks,
                                          const int* open_axes, const int* face_bc,
                                          amps_amr_mesh** out);
/* Constraint rows of the boundary corners: flag[ncorners] (1: boundary row),
 * CSR start[ncorners+1], col/weight[nentries]: row b reads
 * x_b - sum weight x_col = 0.  Any pointer may be NULL. */
amps_gpu_status amps_amr_boundary_tables(const amps_amr_mesh* m, int* nentries, int32_t* flag,
                                         int32_t* start, int32_t* col, double* weight);
/* Leaves of a nested refinement: mode 0 refines a central box of relative
 * half-width frac/2 (halved per level), mode 1 a central sphere of relative
 * radius frac (halved per level); 2:1 balance enforced.  Returns the leaf
 * count (negative status on error) and fills up to cap leaves. */
int amps_amr_nested_leaves(int nbx0, int nby0, int nbz0, int lmax, int mode, double frac,
                           amps_block_desc* out, int cap);

/* ---- context (PIC::Init / ECSIM::Init analogue) ---- */
amps_gpu_status amps_gpu_create(const amps_gpu_config* cfg, amps_gpu_ctx** out);
/* Context on a block-structured AMR mesh (the leaf blocks of the reference's
 * octree, meshAMRgeneric.h): geometry (x0, level-0 dx, level-0 block counts)
 * is taken from the mesh, species/dt/theta/capacity/device from cfg.  Corner
 * fields use the mesh's unique-corner numbering (amps_amr_tables), cell fields
 * block*512 + i + 8j + 64k; a particle's block-local offset is in its block's
 * cell units.  The mesh may be destroyed after this call. */
amps_gpu_status amps_gpu_create_amr(const amps_gpu_config* cfg, const amps_amr_mesh* mesh,
                                    amps_gpu_ctx** out);
/* blocks, cells (block*512 + local) and corners carrying unknowns */
amps_gpu_status amps_gpu_mesh_sizes(const amps_gpu_ctx* ctx, long long* nblocks,
                                    long long* ncells, long long* ncorners);
amps_gpu_status amps_gpu_destroy(amps_gpu_ctx* ctx);
const char* amps_gpu_last_error(const amps_gpu_ctx* ctx);
amps_gpu_status amps_gpu_get_stream(amps_gpu_ctx* ctx, void** stream);
amps_gpu_status amps_gpu_synchronize(amps_gpu_ctx* ctx);

/* ---- PIC::ParticleBuffer import/export (pic.h:2808-3400 accessors) ----
 * x, v: n*3 interleaved FP64; spec: species byte; wcorr: individual weight
 * correction (GetIndividualStatWeightCorrection) or NULL for 1.  The device
 * locates each particle's block and cell with the reference's findTreeNode /
 * FindCellIndex rules and stores FP32 block-local offsets. */
amps_gpu_status amps_gpu_import_particles(amps_gpu_ctx* ctx, long long n, const double* x,
                                          const double* v, const uint8_t* spec,
                                          const double* wcorr);
/* Fast path: block-local FP32 offsets in cell units (x = x0_block + u*dx). */
amps_gpu_status amps_gpu_import_particles_local(amps_gpu_ctx* ctx, long long n, const float* u,
                                                const float* v, const uint8_t* spec,
                                                const int32_t* block);
/* The same with a per-particle weight correction factor (the reference's
 * individual statistical weight correction, GetIndividualStatWeightCorrection
 * pic.h:3438); wcorr may be NULL (all 1). */
amps_gpu_status amps_gpu_import_particles_local_weighted(amps_gpu_ctx* ctx, long long n,
                                                         const float* u, const float* v,
                                                         const uint8_t* spec, const int32_t* block,
                                                         const float* wcorr);
/* Exports in the device order (sorted by block, then cell).  Any pointer may
 * be NULL.  id is the import index when track_ids is set. */
amps_gpu_status amps_gpu_export_particles(amps_gpu_ctx* ctx, double* x, double* v, uint8_t* spec,
                                          int32_t* block, int32_t* cell, uint32_t* id,
                                          long long* n);
amps_gpu_status amps_gpu_num_particles(amps_gpu_ctx* ctx, long long* n);

/* ---- field state (corner E^n, E^{n+theta}; centre B^n; corner B prev/cur) ---- */
amps_gpu_status amps_gpu_import_fields(amps_gpu_ctx* ctx, const double* E_n, const double* E_half,
                                       const double* B_center, const double* B_corner_prev,
                                       const double* B_corner_cur);
/* Where the magnetic field the particles see is interpolated from.  on = 0
 * (default): the corner B slots (_PIC_FIELD_SOLVER_B_CORNER_BASED_).  on = 1:
 * the cell centres (_PIC_FIELD_SOLVER_B_CENTER_BASED_, the reference's default
 * build: Lapenta2017 pic_mover_boris.cpp:979, ProcessCell
 * pic_field_solver_ecsim.cpp:2050-2117, CellCentered::Linear
 * pic_interpolation_routines.cpp:820-905): the push reads B^n, the deposit B^{n+1} (after a
 * field solve; both the imported B_center before the first), E stays at the
 * corners.  Uniform meshes only (INVALID_ARG on AMR).  The no-alloc entry
 * point always reads corner B. */
amps_gpu_status amps_gpu_set_b_center(amps_gpu_ctx* ctx, int on);
amps_gpu_status amps_gpu_export_fields(amps_gpu_ctx* ctx, double* E_n, double* E_half,
                                       double* B_center, double* B_corner_prev,
                                       double* B_corner_cur);
/* J: 3 per corner, M: 243 per corner (global layout above).  Import: uniform
 * meshes only (AMR contexts return AMPS_GPU_INVALID_ARG: their solve reads the
 * per-cell blocks).  Export on AMR contexts: the same corner layout over the
 * mesh's unique corners (J[corner][3], M[corner][243]), each corner the sum of
 * ProcessCell's flush (pic_field_solver_ecsim.cpp:2362-2426) over the cells of
 * any level that have it -- hanging corners included, with their own sums --
 * so an AMR run can take J and M back into its corner nodes.  Either pointer
 * may be NULL.  Page-locked host arrays (cudaHostAlloc / cudaHostRegister)
 * fill at the host link's rate: the AMR corner sums are made in corner ranges
 * whose copies overlap the next range's kernel. */
amps_gpu_status amps_gpu_import_moments(amps_gpu_ctx* ctx, const double* J, const double* M);
amps_gpu_status amps_gpu_export_moments(amps_gpu_ctx* ctx, double* J, double* M);
/* Tecplot ASCII output of the corner fields in the layout of the reference's
 * mesh writer (outputMeshDataTECPLOT, src/meshAMR/meshAMRgeneric.h:8845; data
 * file :7685-7710): VARIABLES "X", "Y", "Z", ECSIM's corner E
 * ("Ex (corner node)" .., pic_field_solver_ecsim.cpp:6416-6420), the corner B
 * ("cur" slot) and E^{n+theta}; one ZONE, DATAPACKING=POINT, ZONETYPE=FEBRICK,
 * one line per corner node (position and values, "%e"), then the 8 node
 * numbers of every cell.  Periodic far faces and AMR corners get nodes at their
 * positions (values of the corner they wrap to / the unique corner). */
amps_gpu_status amps_gpu_write_tecplot(amps_gpu_ctx* ctx, const char* path);

/* div E correction (PIC::FieldSolver::Electromagnetic::ECSIM::divECorrection,
 * src/pic/pic_field_solver_ecsim.cpp:4341-4364; the reference exits when it is
 * switched on, :6168-6170), on periodic uniform meshes -- the reference's own
 * restriction (:4361-4363); other contexts get AMPS_GPU_INVALID_ARG.  After a
 * step (particles at x^{n+1}, E^n the new E): the previous net charge kept as
 * rho_old, the net charge rho_new of the particles on the cell centres
 * (ComputeNetCharge :4690, cell-centred linear weights), div E of the corner E
 * at the centres (ComputeDivE :1474), the Poisson equation Laplacian(phi) =
 * (-4 pi (g rho_new + (1-g) rho_old) + div E) / g, g = 0.51 (PoissonGetStencil
 * :645, PoissonUpdateRhs :6023) solved by CG to ||r|| <= tol ||f|| (the mean
 * of the right-hand side removed: the periodic null space), the species-0
 * positions corrected by -0.9 grad phi / (4 pi rho_e) capped at 0.1 dx
 * (CorrectParticleLocation :4440; rho_e = the species-0 charge density at the
 * nearest corner, summed from the particles) and re-binned, rho_new again.
 * redeposit != 0: then UpdateJMassMatrix on the corrected particles (the
 * reference deposits after the correction).  The densities persist between
 * calls (the first call takes rho_old = rho_new). */
typedef struct {
  int iterations;          /* CG iterations */
  double rel_residual;     /* ||r|| / ||f|| of the Poisson solve */
  double gauss_before;     /* ||div E - 4 pi (g rho_new + (1-g) rho_old)||_2 before ... */
  double gauss_after;      /* ... and after the correction */
  long long moved;         /* species-0 particles corrected */
} amps_gpu_dive_stats;
amps_gpu_status amps_gpu_div_e_correction(amps_gpu_ctx* ctx, double tol, int maxit, int redeposit,
                                          amps_gpu_dive_stats* stats);
/* the per-cell rho_new, rho_old, div E and phi of the last correction (each
 * ncells doubles in the global cell order I + NX (J + NY K) of the field
 * arrays; any may be NULL) */
amps_gpu_status amps_gpu_export_div_e(amps_gpu_ctx* ctx, double* rho_new, double* rho_old,
                                      double* div_e, double* phi);
/* Per-cell pieces of ProcessCell (pic_field_solver_ecsim.cpp:1882-2438) before
 * the corner assembly, cells in block order: cellJ[24] = sum q W w_c (alpha v)
 * for the 8 corners (order (0,0,0),(1,0,0),(1,1,0),(0,1,0), then z+1), and
 * cellM[324] = sum (q W h / V) w_c1 w_c2 alpha (row-major 3x3) for the 36 pairs
 * c2 <= c1.  Accumulated in FP32, returned widened to FP64. */
amps_gpu_status amps_gpu_export_cell_moments(amps_gpu_ctx* ctx, double* cellJ, double* cellM);

/* ---- hot path ---- */
/* PIC::Mover::MoveParticles with Lapenta2017 (pic_mover.cpp:580,
 * pic_mover_boris.cpp:876): E^{n+theta} and the corner B "prev" slot, then
 * re-binning into destination cells (pic_mover.cpp:982-1087, periodic wrap of
 * pic_bc_periodic.cpp:55-178). */
amps_gpu_status amps_gpu_move_particles(amps_gpu_ctx* ctx, long long* out_of_block);
/* Mover::Relativistic::Boris (src/pic/pic_mover_relativistic_boris.cpp:16-583)
 * on the mesh fields: every particle advances by dt_total in FP64 sub-steps of
 * at most one gyro period (1/f_g, f_g = |q||B|/(2 pi m gamma)), with E = the
 * corner E^n slot and B = the corner B "cur" slot interpolated at each
 * sub-step's start, then re-binned.  light_speed in the context's units.
 * Uniform and AMR meshes (on AMR meshes each sub-step re-locates the
 * particle in the block tree and interpolates from its leaf block's corners,
 * hanging corners through their constraint).  A particle past a face of an
 * open axis after a sub-step is deleted (findTreeNode finds no block there).
 * substeps (optional) receives the total sub-steps. */
amps_gpu_status amps_gpu_move_particles_relativistic(amps_gpu_ctx* ctx, double dt_total,
                                                     double light_speed, long long* substeps);
/* PIC::Mover::Boris (src/pic/pic_mover_boris.cpp:126-553, scalar path
 * :264-290), the non-relativistic test-particle mover, with the Lorentz force
 * of BorisSplitAcceleration_default (:104-112): one FP64 step of dt_total per
 * particle, E = the corner E^n slot and B = the corner B "cur" slot
 * interpolated at the particle's start position (CornerBased::InitStencil
 * weights), then re-binning.  Uniform and AMR meshes; a particle past a face
 * of an open axis is deleted (:352-427, the DELETE processing mode). */
amps_gpu_status amps_gpu_move_particles_boris(amps_gpu_ctx* ctx, double dt_total);
/* The per-species CFL number UpdateJMassMatrix reports ("max cfl number for
 * spec", src/pic/pic_field_solver_ecsim.cpp:2236, :2356-2359, :3972-3987): per
 * cell and species sum(|v| dt) / (count * |cell diagonal|), the maximum over
 * the cells that hold the species (cells without it do not count).  Computed
 * on demand from the particles as they are now -- right after a deposition,
 * the particles ProcessCell saw -- in FP64-accurate arithmetic.  cfl[nspec]. */
amps_gpu_status amps_gpu_particle_cfl(amps_gpu_ctx* ctx, double* cfl);
/* ECSIM::UpdateJMassMatrix (pic_field_solver_ecsim.cpp:3244): J and the
 * 243-term mass matrix on all corners from the corner B "cur" slot. */
amps_gpu_status amps_gpu_update_j_mass_matrix(amps_gpu_ctx* ctx, double* particle_energy);
/* ECSIM::TimeStep (pic_field_solver_ecsim.cpp:6179): RHS, GMRES solve for
 * E^{n+theta} = E^n + dE (x0 = 0, stop when ||b-Ax|| <= tol ||b||, restart 30),
 * UpdateB, InterpolateB_C2N, UpdateE.  precond: 0 none (the reference's
 * PrecondParam = 0), 1 Jacobi, 2 the learned block network loaded with
 * amps_gpu_precond_load or trained (Jacobi-scaled input, flexible GMRES).
 * Each restart cycle begins from the FP64 residual b - A x; the Arnoldi steps
 * apply the operator in FP32 unless amps_gpu_set_inner_fp64 switched that off. */
amps_gpu_status amps_gpu_field_solve(amps_gpu_ctx* ctx, double tol, int maxit, int precond,
                                     amps_gpu_solve_stats* stats);
/* One PIC::TimeStep of the ECSIM track (pic_time_step.cpp:403-551): field
 * solve, move, deposit.  Runs UpdateJMassMatrix first if no moments exist yet
 * (the reference's first-call branch, pic_field_solver_ecsim.cpp:6209). */
amps_gpu_status amps_gpu_step(amps_gpu_ctx* ctx, double tol, int maxit, int precond,
                              amps_gpu_step_stats* stats);
/* Particle domain boundaries: an open axis deletes the particles whose move
 * leaves the domain through one of its faces (the mover's
 * _PIC_PARTICLE_DOMAIN_BOUNDARY_INTERSECTION_PROCESSING_MODE__DELETE_ branch,
 * pic_mover_boris.cpp:1159-1170 and :1251-1254, taken when findTreeNode finds
 * no block); the other axes stay periodic (default: all periodic).  The field
 * solve stays periodic on every axis.  deleted_particles: the number deleted
 * since creation (amps_gpu_num_particles drops by as many). */
amps_gpu_status amps_gpu_set_open_axes(amps_gpu_ctx* ctx, int open_x, int open_y, int open_z);
amps_gpu_status amps_gpu_deleted_particles(amps_gpu_ctx* ctx, long long* total);
/* Injection through an open face (the OpenFlow boundary, pic_bc.cpp:270-440),
 * uniform and AMR meshes: every particle step injects on each boundary cell face of
 * `face` (0 -x, 1 +x, 2 -y, 3 +y, 4 -z, 5 +z; its axis must be open) the
 * particles of species `spec` that a Maxwellian of number density `density`,
 * bulk velocity drift[3] (NULL: 0) and thermal speed vth = sqrt(kT/m) sends
 * through it in dt (CalculateInjectionRate_MaxwellianDistribution,
 * pic_bc.cpp:215, / the species weight): Poisson arrivals in time, uniform on
 * the face, velocity from InjectMaxwellianDistribution
 * (pic_vel_distribution.cpp:49), moved by the mover for the rest of the step
 * and deposited with the others.  Up to 8 sources.  Random numbers come from
 * counter-based streams keyed by the seed, the step, the source and the face
 * cell (AMR meshes: the finest-lattice face patch); injected particles get
 * ids after the imported ones. */
amps_gpu_status amps_gpu_add_injection(amps_gpu_ctx* ctx, int face, int spec, double density,
                                       const double* drift, double vth);
amps_gpu_status amps_gpu_clear_injection(amps_gpu_ctx* ctx);
amps_gpu_status amps_gpu_set_injection_seed(amps_gpu_ctx* ctx, unsigned long long seed);
amps_gpu_status amps_gpu_injected_particles(amps_gpu_ctx* ctx, long long* total);
/* Species moments on corners (_PIC_FIELD_SOLVER_SAMPLE_SPECIES_ON_CORNER_,
 * ProcessCell pic_field_solver_ecsim.cpp:2270-2303): with sampling on, every
 * deposition (update_j_mass_matrix, push_deposit, step) also forms per corner
 * and species rho, rho u (3), rho u u (xx, yy, zz, xy, yz, xz) of the
 * particles after the step, each cell's sums divided by its volume (the
 * SpecData flush :2384-2394).  Export: out[corner][10*nspec] in the
 * reference's Rho_ .. RhoUxUz_ order, corners in the fields' corner order (on
 * AMR meshes hanging corners carry the sums of the fine cells that have them
 * as a corner). */
amps_gpu_status amps_gpu_set_species_moments(amps_gpu_ctx* ctx, int on);
amps_gpu_status amps_gpu_export_species_moments(amps_gpu_ctx* ctx, double* out);

/* Particle record of the caller's build (picParticleBasicOffset.cpp:160-200):
 * its length (ParticleDataLength) and the byte offsets of the velocity
 * (3 double), position (3 double), species (unsigned char) and weight
 * correction (double; -1 when the build has none).  The first 16 bytes are the
 * next/prev list links.  Basic build: {65, 16, 40, 64, -1}; with the weight
 * correction {80, 16, 40, 64, 72} (8-byte alignment of the offset). */
typedef struct {
  int record_length;
  int off_velocity;
  int off_position;
  int off_species;
  int off_weight;
} amps_gpu_record_layout;
/* Particle section of a restart file (PIC::Restart::SaveParticleData,
 * pic_restart.cpp:248-310, SaveParticleDataBlock :312-382): the end-of-user-
 * data marker, ParticleDataLength (long int), the species weights, then for
 * each block holding particles, in block_order (NULL: block index order; the
 * reference's tree order is the caller's), its node id (id_length bytes taken
 * from node_ids[block*id_length], the caller's cAMRnodeID), the count, the
 * ParticleNumberTable[i][j][k] and the records of cells i, j, k in reverse
 * list order.  List links are written as zero; fields the device does not
 * hold are zero.  Records are packed on the device; out is host memory of at
 * least restart_particle_bytes(). */
amps_gpu_status amps_gpu_restart_particle_bytes(amps_gpu_ctx* ctx, const amps_gpu_record_layout* layout,
                                                int id_length, long long* bytes);
amps_gpu_status amps_gpu_write_restart_particles(amps_gpu_ctx* ctx, const amps_gpu_record_layout* layout,
                                                 const int32_t* block_order, const void* node_ids,
                                                 int id_length, void* out, long long capacity,
                                                 long long* written);
/* PIC::Restart::ReadParticleData (pic_restart.cpp:515-575,
 * ReadParticleDataBlock :430-512): replaces the particles by those of a
 * particle section (node ids mapped to blocks through node_ids), each cell in
 * the list order it had when saved; the species weights are taken from the
 * section.  Unpacked on the device.  A record whose position lies outside the
 * cell of its table entry, or whose species is out of range, is counted and
 * reported as AMPS_GPU_INVALID_ARG after loading (position clamped into the
 * cell, species 0). */
amps_gpu_status amps_gpu_read_restart_particles(amps_gpu_ctx* ctx, const amps_gpu_record_layout* layout,
                                                const void* data, long long size, const void* node_ids,
                                                int id_length, long long* nread);
/* PIC::Restart::GetParticleDataCheckSum (pic_restart.cpp:578-660): the CRC32
 * class of specfunc.h:438-505 (polynomial 0x04C11DB7, initial value 0, its
 * 64-bit accumulator) over every particle record with zeroed links
 * (GetParticleSignature, pic_pbuffer.cpp:1109-1123), blocks in block_order,
 * cells i, j, k, list order.  Per-record CRCs are formed on the device and
 * combined with the CRC append operator. */
amps_gpu_status amps_gpu_particle_checksum(amps_gpu_ctx* ctx, const amps_gpu_record_layout* layout,
                                           const int32_t* block_order, unsigned long long* checksum);
/* Particle push + re-bin + deposit only (the particle-steps/s hot path). */
amps_gpu_status amps_gpu_push_deposit(amps_gpu_ctx* ctx, double* particle_energy);
/* GMRES inner operator precision: 0 FP32 arithmetic with FP64 refinement at
 * each restart (default), 1 FP64 throughout.  No reference counterpart (the
 * reference's solve is FP64). */
amps_gpu_status amps_gpu_set_inner_fp64(amps_gpu_ctx* ctx, int fp64);

/* ---- learned right preconditioner for the field solve (no reference
 *      counterpart: the reference's GMRES takes PrecondParam 0/1 only) ----
 * Network, per mesh block: input x = D r (Jacobi-scaled residual) on the
 * block's 8^3 owned corners plus a 1-corner halo (10^3 corners, 3 channels),
 * three 3x3x3 convolutions 3 -> 32 -> 32 -> 3 with zero padding at the halo
 * edge and no activation, output on the owned corners; z = x + N(x).
 * Weights: w1[27][3][32], w2[27][32][32], w3[27][32][3] (tap t = (dx+1) +
 * 3(dy+1) + 9(dz+1), then input channel, then output channel), FP32 masters,
 * BF16 copies for inference.  Training pairs come from the Jacobi field solves
 * themselves (harvest on): each Arnoldi step's (r = A e, e) and the final
 * (b, x), cut into blocks and normalised by the RMS of D r over the block.
 * On AMR meshes the halo corners are those of the block's own lattice (zero
 * where a coarser neighbour has none, and at hanging corners), a free corner
 * is written by the block whose cell has it as low corner, hanging corners
 * get z = D r, and every refinement level has its own weight set. */
/* weight sets: 1 on a uniform mesh, lmax + 1 on an AMR mesh (set = level).
 * load, get, train, loss_grad and forward act on the selected set (0 at
 * creation); inference inside the field solve uses each block's own set. */
amps_gpu_status amps_gpu_precond_num_sets(amps_gpu_ctx* ctx, int* n);
amps_gpu_status amps_gpu_precond_select(amps_gpu_ctx* ctx, int set);
/* on != 0: blocks whose halo region reaches a refinement interface (a hanging
 * corner, or a position with no corner of the block's lattice) use Jacobi
 * instead of the network, and training skips their samples; *nblocks (may be
 * NULL) receives their number. */
amps_gpu_status amps_gpu_precond_interface_jacobi(amps_gpu_ctx* ctx, int on, int* nblocks);
amps_gpu_status amps_gpu_precond_load(amps_gpu_ctx* ctx, const float* w1, const float* w2,
                                      const float* w3);
amps_gpu_status amps_gpu_precond_get(amps_gpu_ctx* ctx, float* w1, float* w2, float* w3);
/* inference path used inside the field solve: 1 BF16 tcgen05 kernel, 0 FP32
 * training forward (default after load: 0) */
amps_gpu_status amps_gpu_precond_use_tensor_cores(amps_gpu_ctx* ctx, int on);
/* enable (capacity > 0: keep up to capacity block samples) or stop harvesting */
amps_gpu_status amps_gpu_precond_harvest(amps_gpu_ctx* ctx, long long capacity);
amps_gpu_status amps_gpu_precond_num_samples(amps_gpu_ctx* ctx, long long* n);
/* read samples [first, first+count): x[count][1000][3] (halo region, z-major:
 * index (k*10 + j)*10 + i for block corner (i-1, j-1, k-1)), e[count][512][3] */
amps_gpu_status amps_gpu_precond_get_samples(amps_gpu_ctx* ctx, long long first, long long count,
                                             float* x, float* e);
/* weight set (block level) of samples [first, first+count) */
amps_gpu_status amps_gpu_precond_sample_sets(amps_gpu_ctx* ctx, long long first, long long count,
                                             int32_t* sets);
/* Adam on the harvested samples of the selected weight set (mini-batches of
 * `batch` blocks, shuffled with `seed`); loss = mean over owned corners and
 * channels of (x + N(x) - e)^2.
 * loss_out[epochs] receives the mean loss of every epoch. */
amps_gpu_status amps_gpu_precond_train(amps_gpu_ctx* ctx, int epochs, int batch, float lr,
                                       unsigned long long seed, float* loss_out);
/* Loss and weight gradients of the current weights on given samples (host
 * arrays in the get_samples layout), computed by the training kernels. */
amps_gpu_status amps_gpu_precond_loss_grad(amps_gpu_ctx* ctx, long long count, const float* x,
                                           const float* e, float* loss, float* g1, float* g2,
                                           float* g3);
/* N(x) on given samples by the inference path (tensor_cores 1: BF16 tcgen05
 * kernel; 0: the FP32 training forward).  y[count][512][3]. */
amps_gpu_status amps_gpu_precond_forward(amps_gpu_ctx* ctx, long long count, const float* x,
                                         int tensor_cores, float* y);

/* ---- deposition for callers that may not allocate device memory ----
 * No counterpart in the reference: a variant of UpdateJMassMatrix for a host
 * code that may not call cudaMalloc or cudaFree through a library -- its
 * device memory belongs to its framework's pool allocator, or it must not
 * stall its other streams in mid-step (cudaFree synchronises the device).  It
 * allocates nothing: the caller passes device buffers for every input and
 * output, and the block stencils and per-cell partial sums in between live in
 * one static device array of 11.1 MiB that every GPU loading the library keeps
 * until exit.  That array limits the mesh to 16 blocks (8192 cells); larger
 * meshes return AMPS_GPU_INVALID_ARG.  All calls share it, so calls that
 * overlap on the GPU race; each call writes the scratch it reads before
 * reading it, so nothing carries over between calls.  The first call on a
 * device looks up the array's address (cudaGetSymbolAddress), which must not
 * run while a stream of that device is being captured.  The caller's current
 * device is restored on return.
 * Inputs (device pointers, asynchronous on `stream`): particles sorted by cell
 * key block*512 + (i + 8*(j + 8*k)), d_cell_start[ncell+1] their offsets; d_u,
 * d_v structure-of-arrays of length 3n (x[n], y[n], z[n]) with u the FP32
 * block-local offset in cell units; d_spec species bytes; d_B_corner the corner
 * B "cur" slot, 3 per corner in the global layout.  Outputs: d_J (3 per corner),
 * d_M (243 per corner) in the global layout, d_energy[1] the kinetic energy.
 * If the device hit a bounded-wait timeout, *d_energy is NaN and the J and M
 * entries the affected blocks contribute to are NaN: treat J and M as invalid
 * whenever *d_energy is NaN.  cfg->device selects the GPU; particle_capacity
 * and track_ids are ignored. */
amps_gpu_status amps_gpu_update_j_mass_matrix_noalloc(const amps_gpu_config* cfg, long long n,
                                                      const int32_t* d_cell_start,
                                                      const float* d_u, const float* d_v,
                                                      const uint8_t* d_spec,
                                                      const double* d_B_corner, double* d_J,
                                                      double* d_M, double* d_energy,
                                                      void* stream);

/* ---- launch configuration (no reference counterpart) ----
 * set_graphs: run the particle step (flag reset, stencil pack, push/deposit,
 * arrivals, assembly, flag read-back) as a captured CUDA graph, one per set of
 * field buffers it reads; graphs are not used while kernel timing is on.
 * autotune: times 3 CTA sizes of the field operator kernels and 3 grid sizes of
 * the GMRES sweeps on this context's data and keeps the fastest; ms[6]
 * (optional) receives the candidates' times. get_tuning reads the choice. */
amps_gpu_status amps_gpu_set_graphs(amps_gpu_ctx* ctx, int on);
amps_gpu_status amps_gpu_autotune(amps_gpu_ctx* ctx, double* ms);
amps_gpu_status amps_gpu_get_tuning(amps_gpu_ctx* ctx, int* threads_per_cta, int* reduction_ctas);
/* The particle side of the autotuner: amps_gpu_autotune also arms a
 * comparison of the arrivals kernel staging 16 or 32 arrivals at a time over
 * the next 6 particle steps (3 each, stream launches timed by events; the
 * steps do their work as usual), then keeps the faster.  get: the chunk in use,
 * the steps still to compare, ms[2] mean ms per launch of each (0 until
 * measured).  set: force one (16 or 32), ending a comparison. */
amps_gpu_status amps_gpu_set_arrivals_chunk(amps_gpu_ctx* ctx, int chunk);
amps_gpu_status amps_gpu_get_particle_tuning(amps_gpu_ctx* ctx, int* arrivals_chunk, int* pending,
                                             double* ms);

/* ---- per-kernel device timing on the context stream (CUDA events) ---- */
amps_gpu_status amps_gpu_set_kernel_timing(amps_gpu_ctx* ctx, int enable);
/* Fills up to cap entries; names are static strings.  Returns the count in *n. */
amps_gpu_status amps_gpu_get_kernel_times(amps_gpu_ctx* ctx, const char** names, double* total_ms,
                                          long long* launches, int cap, int* n);
amps_gpu_status amps_gpu_reset_kernel_times(amps_gpu_ctx* ctx);

/* ---- host-side initial condition (test/srcFastWave/main.cpp:270-300 style) ----
 * Uniform positions in every cell and Maxwellian velocities (Box-Muller on the
 * reference LCG of src/general/rnd.h:56-77), one co-located particle of every
 * species per draw.  Outputs are FP32-representable so an FP64 consumer and
 * the FP32 device start from identical particles.  Sizes: n = ncells*ppc*nspec.
 * u: block-local offsets in cell units (3 per particle), v: 3 per particle,
 * block: block id.  Draws are jump-ahead seeded per block and generated with
 * nthreads host threads (result independent of nthreads). */
long long amps_ic_count(int nbx, int nby, int nbz, int ppc, int nspec);
int amps_ic_maxwellian(int nbx, int nby, int nbz, int ppc, int nspec, const double* vth,
                       unsigned long long seed, int nthreads, float* u, float* v, uint8_t* spec,
                       int32_t* block);

/* ---- batched relativistic test-particle tracing (config: dipole + uniform) ----
 * BorisStep of srcEarth/gridless/GridlessParticleMovers.cpp:781 with the
 * gyro-angle limiter dt = min(dt_max, dphi_max/omega) of
 * CutoffRigidityGridless.cpp:1190-1197, one persistent kernel with warp-level
 * compaction of finished particles.  SI units.  x, p: n*3 host arrays updated
 * in place; status: 1 r<r_in, 2 r>r_out, 0 step cap; steps: steps taken.
 * precision: 0 FP64, 1 FP32.  total_steps receives the sum of steps. */
amps_gpu_status amps_gpu_trace_dipole(int device, long long n, double* x, double* p,
                                      int32_t* status, int64_t* steps, double q, double m0,
                                      double b_eq, double r_e, const double* b_ext, double r_in,
                                      double r_out, long long max_steps, double dphi_max,
                                      double dt_max, int precision, long long* total_steps,
                                      double* kernel_ms);

#ifdef __cplusplus
}
#endif
#endif
