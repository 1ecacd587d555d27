// Golden vectors from the reference's own ECSIM particle routines, compiled
// from the reference tree (test infrastructure: the output pins the FP64
// oracle, tests/test_oracle_pins.py).
//
// Compiled with this harness (oracle/Makefile, target ref):
//   src/pic/pic_field_solver_ecsim.cpp      ECSIM::ProcessCell (:1882-2438)
//   src/pic/pic_mover_boris.cpp             Mover::Lapenta2017 (:876-1380),
//                                           Mover::Boris (:126-553)
//   src/pic/pic_interpolation_routines.cpp  CornerBased::InitStencil (:1074-1194)
// against the hand-written configuration pins/refcfg/general.conf (ECSIM,
// corner B, normalised units, one global time step, one species slot) and
// declaration-only stand-ins for MPI and the SWMF coupler (pins/refcfg/).
//
// The functions run on one block of the reference's default 5^3 cells (2
// ghost layers) at origin 0 with cell size dx; the harness builds that block,
// its corner nodes and the particle buffer directly (no mesh generation), and
// defines the few globals the functions read.  Particles stay inside the
// block, so findTreeNode returns the block itself.  pic.h fixes the species
// count at 1 without its configuration script, so every call runs with the
// electron (q -1, m 1) or the proton (q +1, m 25) in species slot 0; the
// "species" field of each record says which.
//
// Built with PIN_B_CENTER (oracle/_ref/ecsim_pin_cb), the configuration puts
// the magnetic field on the cell centres (_PIC_FIELD_SOLVER_B_CENTER_BASED_,
// the reference's default) with the cell-centred linear interpolation: the
// block then also gets its centre nodes (ghost layers included) carrying B in
// the current and previous slots, Lapenta2017's B_C scratch holds the centre
// values, and the record adds "b_mode": "center" and "center_fields" (B at the
// centres of cells 0..4).  CellCentered::Linear::InitStencil reads the global
// StencilTable[0].Length to decide whether to renormalise its weights
// (pic_interpolation_routines.cpp:900): it is set to 8, a full stencil, so the
// weights are used as computed.
//
// Output (JSON on stdout):
//   process_cell: cells with particles (x, v, species, weight correction) and
//     the 8 corners' J[3] and M[243] of ProcessCell's CellData plus the cell's
//     ParticleEnergy and cflCell;
//   lapenta: particles with corner fields E^{n+theta}, B, and x', v' after
//     Lapenta2017;
//   boris: the same for Mover::Boris, whose force hook
//     (_PIC_PARTICLE_MOVER__BORIS_SPLIT_ACCELERATION_) is set to
//     pin_boris_split_acceleration: E and B of the corner fields at x with the
//     reference's CornerBased::InitStencil weights, accl = (q/m) E,
//     rotation = -(q/m) B, as BorisSplitAcceleration_default (:104-112);
//   fields, corner_fields: the corner field function and its values at the
//     corners of the block's cells, used for both.
#include "pic.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <new>
#include <vector>

// ---- globals the compiled functions read, defined elsewhere in AMPS ----
MPI_Comm MPI_GLOBAL_COMMUNICATOR = 0;
double PIC::MolecularData::MolMass[_TOTAL_SPECIES_NUMBER_];
double PIC::MolecularData::ElectricChargeTable[_TOTAL_SPECIES_NUMBER_];
long int PIC::ParticleBuffer::ParticleDataLength = 0;
PIC::ParticleBuffer::byte* PIC::ParticleBuffer::ParticleDataBuffer = nullptr;
double PIC::ParticleWeightTimeStep::GlobalParticleWeight[_TOTAL_SPECIES_NUMBER_];
double PIC::ParticleWeightTimeStep::GlobalTimeStep[_TOTAL_SPECIES_NUMBER_];
PIC::CPLR::DATAFILE::cOffsetElement PIC::CPLR::DATAFILE::Offset::ElectricField;
PIC::CPLR::DATAFILE::cOffsetElement PIC::CPLR::DATAFILE::Offset::MagneticField;
cMeshAMR3d<PIC::Mesh::cDataCornerNode, PIC::Mesh::cDataCenterNode, PIC::Mesh::cDataBlockAMR>*
    PIC::Mesh::mesh = nullptr;
picunits::Factors PIC::Units::Factors;

// species-dependent global particle weight (the _SPECIES_DEPENDENT_GLOBAL_
// branch of the reference accessor in src/pic/pic.cpp)
double PIC::Mesh::cDataBlockAMR::GetLocalParticleWeight(int spec) {
  return PIC::ParticleWeightTimeStep::GlobalParticleWeight[spec];
}

// the reference's error exit: report and stop
void exit(long int line, const char* file, const char* msg) {
  fprintf(stderr, "reference exit at %s:%ld: %s\n", file, line, msg ? msg : "");
  std::abort();
}

PIC::ParticleBuffer::byte* PIC::ParticleBuffer::GetParticleDataPointer(long int ptr) {
  return ParticleDataBuffer + ptr * ParticleDataLength;
}

namespace {
const double* g_hook_E = nullptr;  // corner fields the Boris force hook reads
const double* g_hook_B = nullptr;
}  // namespace

void pin_boris_split_acceleration(double* accl, double* rotation, int spec, long int, double* x,
                                  double*, void* startNode) {
  PIC::InterpolationRoutines::CornerBased::cStencil st;
  PIC::InterpolationRoutines::CornerBased::InitStencil(
      x, static_cast<cTreeNodeAMR<PIC::Mesh::cDataBlockAMR>*>(startNode), st);
  double E[3] = {0, 0, 0}, B[3] = {0, 0, 0};
  for (int t = 0; t < st.Length; t++)
    for (int d = 0; d < 3; d++) {
      E[d] += st.Weight[t] * g_hook_E[3 * st.LocalCellID[t] + d];
      B[d] += st.Weight[t] * g_hook_B[3 * st.LocalCellID[t] + d];
    }
  const double qm = PIC::MolecularData::GetElectricCharge(spec) / PIC::MolecularData::GetMass(spec);
  for (int d = 0; d < 3; d++) {
    accl[d] = 0.0 + qm * E[d];
    rotation[d] = 0.0 - qm * B[d];
  }
}

namespace {

using Node = cTreeNodeAMR<PIC::Mesh::cDataBlockAMR>;
namespace EC = PIC::FieldSolver::Electromagnetic::ECSIM;

constexpr int NX = _BLOCK_CELLS_X_;
constexpr int NG = _GHOST_CELLS_X_;
#if _PIC_FIELD_SOLVER_B_MODE_ == _PIC_FIELD_SOLVER_B_CENTER_BASED_
constexpr bool kCenterB = true;
#else
constexpr bool kCenterB = false;
#endif
constexpr int NCEN = _TOTAL_BLOCK_CELLS_X_ * _TOTAL_BLOCK_CELLS_Y_ * _TOTAL_BLOCK_CELLS_Z_;
constexpr int NCOR = (1 + _TOTAL_BLOCK_CELLS_X_) * (1 + _TOTAL_BLOCK_CELLS_Y_) * (1 + _TOTAL_BLOCK_CELLS_Z_);
// corner associated data: E^n[3] E^{n+theta}[3] J[3] M[243] | B cur[3] B prev[3]
constexpr int kRecDoubles = 258;

// reference LCG of src/general/rnd.h (seed * 48828125 mod 2^31), as doubles
struct Lcg {
  unsigned long long s;
  double next() {
    s = (s * 48828125ULL) & 0x7FFFFFFFULL;
    if (s == 0) s = 1;
    return (double)s / 2147483648.0;
  }
};

// smooth corner fields: f_c(x) = a_c + sum_d b_cd sin(k_d x_d + p_cd)
struct FieldFn {
  double a[6], b[6][3], p[6][3], k[3];
  double at(int comp, const double x[3]) const {
    double v = a[comp];
    for (int d = 0; d < 3; d++) v += b[comp][d] * std::sin(k[d] * x[d] + p[comp][d]);
    return v;
  }
};

struct Block {
  Node* node;
  PIC::Mesh::cDataBlockAMR* block;
  std::vector<PIC::Mesh::cDataCornerNode*> corners;
  std::vector<double> assoc;   // kRecDoubles per corner
  std::vector<double> E, B;    // 3 per corner local number (Lapenta2017 scratch)
  std::vector<double> cassoc;  // centre B: current[3] previous[3] per centre node
  std::vector<double> Bcen;    // 3 per centre local number (Lapenta2017 scratch, centre B)
  double dx;
};

void corner_position(double dx, int nd, double x[3]) {
  const int n1 = 1 + _TOTAL_BLOCK_CELLS_X_;
  const int i = nd % n1 - NG, j = (nd / n1) % n1 - NG, k = nd / (n1 * n1) - NG;
  x[0] = i * dx;
  x[1] = j * dx;
  x[2] = k * dx;
}

Block make_block(double dx, const FieldFn& f) {
  Block b;
  b.dx = dx;
  auto* m = static_cast<decltype(PIC::Mesh::mesh)>(calloc(1, sizeof(*PIC::Mesh::mesh)));
  for (int d = 0; d < 3; d++) {
    m->xGlobalMin[d] = 0.0;
    m->dx_max_refinment[d] = dx;
    m->dxRootBlock[d] = NX * dx;
  }
  // the one non-trivial member the pinned functions touch (Boris walks the
  // internal-boundary list): construct it in place, empty
  using BoundaryList = decltype(m->InternalBoundaryList);
  new (&m->InternalBoundaryList) BoundaryList();
  PIC::Mesh::mesh = m;
  b.node = static_cast<Node*>(calloc(1, sizeof(Node)));
  b.block = static_cast<PIC::Mesh::cDataBlockAMR*>(calloc(1, sizeof(PIC::Mesh::cDataBlockAMR)));
  for (int d = 0; d < 3; d++) {
    b.node->xmin[d] = 0.0;
    b.node->xmax[d] = NX * dx;
    b.node->xMinGlobalIndex[d] = 0;
  }
  b.node->NodeGeometricSizeIndex = NX;
  b.node->RefinmentLevel = 0;
  b.node->IsUsedInCalculationFlag = true;
  b.node->block = b.block;
  for (int c = 0; c < NX * NX * NX; c++) {
    b.block->FirstCellParticleTable[c] = -1;
    b.block->tempParticleMovingListTable[c] = -1;
  }
  b.assoc.assign((size_t)NCOR * kRecDoubles, 0.0);
  b.E.assign(3 * NCOR, 0.0);
  b.B.assign(3 * NCOR, 0.0);
  b.corners.resize(NCOR);
  for (int nd = 0; nd < NCOR; nd++) {
    auto* cn = static_cast<PIC::Mesh::cDataCornerNode*>(calloc(1, sizeof(PIC::Mesh::cDataCornerNode)));
    cn->associatedDataPointer = reinterpret_cast<char*>(&b.assoc[(size_t)nd * kRecDoubles]);
    b.corners[nd] = cn;
    b.block->GetCornerNodeBuffer()[nd] = cn;
    double x[3];
    corner_position(dx, nd, x);
    double* r = &b.assoc[(size_t)nd * kRecDoubles];
    for (int q = 0; q < 3; q++) {
      b.E[3 * nd + q] = f.at(q, x);
      b.B[3 * nd + q] = f.at(3 + q, x);
      r[3 + q] = b.E[3 * nd + q];      // E^{n+theta}
      r[252 + q] = b.B[3 * nd + q];    // corner B, current slot
      r[255 + q] = b.B[3 * nd + q];    // corner B, previous slot
    }
  }
  if (kCenterB) {
    b.cassoc.assign((size_t)NCEN * 6, 0.0);
    b.Bcen.assign((size_t)NCEN * 3, 0.0);
    for (int k = -NG; k < NX + NG; k++)
      for (int j = -NG; j < NX + NG; j++)
        for (int i = -NG; i < NX + NG; i++) {
          const int nd = _getCenterNodeLocalNumber(i, j, k);
          auto* cn = static_cast<PIC::Mesh::cDataCenterNode*>(calloc(1, sizeof(PIC::Mesh::cDataCenterNode)));
          cn->associatedDataPointer = reinterpret_cast<char*>(&b.cassoc[(size_t)nd * 6]);
          b.block->GetCenterNodeBuffer()[nd] = cn;
          const double x[3] = {(i + 0.5) * dx, (j + 0.5) * dx, (k + 0.5) * dx};
          for (int q = 0; q < 3; q++) {
            const double v = f.at(3 + q, x);
            b.cassoc[(size_t)nd * 6 + q] = v;      // CurrentBOffset 0
            b.cassoc[(size_t)nd * 6 + 3 + q] = v;  // PrevBOffset 3 doubles
            b.Bcen[(size_t)nd * 3 + q] = v;
          }
        }
  }
  return b;
}

struct Particle {
  double x[3], v[3], w;
  int s;
};

void put(PIC::ParticleBuffer::byte* p, const Particle& q, long next, long prev) {
  PIC::ParticleBuffer::SetI(q.s, p);
  PIC::ParticleBuffer::SetV(const_cast<double*>(q.v), p);
  PIC::ParticleBuffer::SetX(const_cast<double*>(q.x), p);
  PIC::ParticleBuffer::SetIndividualStatWeightCorrection(q.w, p);
  PIC::ParticleBuffer::SetNext(next, p);
  PIC::ParticleBuffer::SetPrev(prev, p);
}

void print_particle(const Particle& q) {
  printf("{\"x\":[%.17g,%.17g,%.17g],\"v\":[%.17g,%.17g,%.17g],\"spec\":%d,\"wcorr\":%.17g}", q.x[0],
         q.x[1], q.x[2], q.v[0], q.v[1], q.v[2], q.s, q.w);
}

}  // namespace

int main() {
  // plasma of the ECSIM workloads: electrons (q -1, m 1) and protons (q +1,
  // m 25), weight dx^3 / (4 pi ppc) at ppc 16, dt 0.1, dx 1
  const double dx = 1.0, dt = 0.1;
  const double w = dx * dx * dx / (4.0 * M_PI * 16.0);
  const double q_of[2] = {-1.0, 1.0}, m_of[2] = {1.0, 25.0};
  auto use_species = [&](int s) {
    PIC::MolecularData::ElectricChargeTable[0] = q_of[s];
    PIC::MolecularData::MolMass[0] = m_of[s];
  };
  PIC::ParticleWeightTimeStep::GlobalParticleWeight[0] = w;
  PIC::ParticleWeightTimeStep::GlobalTimeStep[0] = dt;
  PIC::Units::Factors.Si2NoM = 1.0;
  PIC::Units::Factors.Si2NoQ = 1.0;
  PIC::CPLR::DATAFILE::Offset::ElectricField.RelativeOffset = 0;
  PIC::CPLR::DATAFILE::Offset::MagneticField.RelativeOffset = 0;
  EC::dtTotal = dt;  // set by the reference's ECSIM::Init from GlobalTimeStep[0] (:557-561)
  EC::JxOffsetIndex = 6;
  EC::MassMatrixOffsetIndex = 9;
  EC::OffsetB_corner = 252 * (int)sizeof(double);
  EC::CurrentBOffset = 0;
  EC::PrevBOffset = 3 * (int)sizeof(double);

  Lcg rng{12345};
  FieldFn f;
  for (int d = 0; d < 3; d++) f.k[d] = 2.0 * M_PI / (8.0 * dx);
  for (int c = 0; c < 6; c++) {
    f.a[c] = (c < 3 ? 0.02 : 0.2) * (2.0 * rng.next() - 1.0);
    for (int d = 0; d < 3; d++) {
      f.b[c][d] = (c < 3 ? 0.01 : 0.1) * rng.next();
      f.p[c][d] = 2.0 * M_PI * rng.next();
    }
  }
  f.a[5] += 0.5;  // B0 along z
  Block blk = make_block(dx, f);
  static PIC::InterpolationRoutines::CellCentered::cStencil stencil_table[1];
  stencil_table[0].Length = 8;
  PIC::InterpolationRoutines::CellCentered::StencilTable = stencil_table;

  const int L = _PIC_PARTICLE_DATA__BASIC_DATA_LENGTH_;
  PIC::ParticleBuffer::ParticleDataLength = L;
  std::vector<PIC::ParticleBuffer::byte> buf((size_t)L * 4096, 0);
  PIC::ParticleBuffer::ParticleDataBuffer = buf.data();

  printf("{\"block_cells\":%d,\"dx\":%.17g,\"dt\":%.17g,\"weight\":%.17g,", NX, dx, dt, w);
  printf("\"charge\":[-1,1],\"mass\":[1,25],\"species_names\":[\"electron\",\"proton\"],");
  printf("\"fields\":{\"a\":[");
  for (int c = 0; c < 6; c++) printf("%s%.17g", c ? "," : "", f.a[c]);
  printf("],\"b\":[");
  for (int c = 0; c < 6; c++)
    for (int d = 0; d < 3; d++) printf("%s%.17g", (c || d) ? "," : "", f.b[c][d]);
  printf("],\"p\":[");
  for (int c = 0; c < 6; c++)
    for (int d = 0; d < 3; d++) printf("%s%.17g", (c || d) ? "," : "", f.p[c][d]);
  printf("],\"k\":[%.17g,%.17g,%.17g]},", f.k[0], f.k[1], f.k[2]);
  // the corner values of the block's cells (corners 0..NX per axis, i fastest):
  // E^{n+theta}[3] then B[3]
  printf("\"corner_fields\":[");
  for (int k = 0; k <= NX; k++)
    for (int j = 0; j <= NX; j++)
      for (int i = 0; i <= NX; i++) {
        const int nd = _getCornerNodeLocalNumber(i, j, k);
        printf("%s[%.17g,%.17g,%.17g,%.17g,%.17g,%.17g]", (i || j || k) ? "," : "", blk.E[3 * nd],
               blk.E[3 * nd + 1], blk.E[3 * nd + 2], blk.B[3 * nd], blk.B[3 * nd + 1], blk.B[3 * nd + 2]);
      }
  printf("],");
  if (kCenterB) {
    // B at the centres of cells 0..NX-1 (i fastest)
    printf("\"b_mode\":\"center\",\"center_fields\":[");
    for (int k = 0; k < NX; k++)
      for (int j = 0; j < NX; j++)
        for (int i = 0; i < NX; i++) {
          const int nd = _getCenterNodeLocalNumber(i, j, k);
          printf("%s[%.17g,%.17g,%.17g]", (i || j || k) ? "," : "", blk.Bcen[3 * nd], blk.Bcen[3 * nd + 1],
                 blk.Bcen[3 * nd + 2]);
        }
    printf("],");
  }

  // ---- ProcessCell on three cells of the block interior ----
  const int cells[4][3] = {{1, 2, 3}, {2, 2, 2}, {3, 1, 2}, {2, 3, 1}};
  const int counts[4] = {37, 64, 5, 48};
  long next_free = 0;
  printf("\"process_cell\":[");
  for (int t = 0; t < 4; t++) {
    const int species = t % 2;
    use_species(species);
    const int ci = cells[t][0], cj = cells[t][1], ck = cells[t][2];
    std::vector<Particle> ps(counts[t]);
    long head = -1;
    for (int n = 0; n < counts[t]; n++) {
      Particle& q = ps[n];
      q.x[0] = (ci + rng.next()) * dx;
      q.x[1] = (cj + rng.next()) * dx;
      q.x[2] = (ck + rng.next()) * dx;
      q.s = 0;
      const double vt = species ? 0.01 : 0.05;
      for (int d = 0; d < 3; d++) q.v[d] = vt * (2.0 * rng.next() - 1.0) * 1.7;
      q.w = 0.5 + 1.5 * rng.next();
      const long ptr = next_free++;
      put(buf.data() + ptr * L, q, head, -1);
      if (head != -1) PIC::ParticleBuffer::SetPrev(ptr, buf.data() + head * L);
      head = ptr;
    }
    blk.block->FirstCellParticleTable[ci + NX * (cj + NX * ck)] = head;
    EC::cCellData cd;
    cd.clean();
    EC::cProcessCellData pd;
    EC::ProcessCell(ci, cj, ck, blk.node, &cd, 0, 1, PIC::MolecularData::MolMass,
                    PIC::MolecularData::ElectricChargeTable, L, buf.data(), pd);
    // the list order ProcessCell walked: head first
    printf("%s{\"species\":%d,\"cell\":[%d,%d,%d],\"particles\":[", t ? "," : "", species, ci, cj, ck);
    long p = head;
    bool first = true;
    while (p != -1) {
      PIC::ParticleBuffer::byte* pp = buf.data() + p * L;
      Particle q;
      PIC::ParticleBuffer::GetX(q.x, pp);
      PIC::ParticleBuffer::GetV(q.v, pp);
      q.s = PIC::ParticleBuffer::GetI(pp);
      q.w = PIC::ParticleBuffer::GetIndividualStatWeightCorrection(pp);
      if (!first) printf(",");
      print_particle(q);
      first = false;
      p = PIC::ParticleBuffer::GetNext(pp);
    }
    printf("],\"J\":[");
    for (int c = 0; c < 8; c++)
      for (int q = 0; q < 3; q++) printf("%s%.17g", (c || q) ? "," : "", cd.CornerData[c].CornerJ[q]);
    printf("],\"M\":[");
    for (int c = 0; c < 8; c++)
      for (int q = 0; q < 243; q++)
        printf("%s%.17g", (c || q) ? "," : "", cd.CornerData[c].CornerMassMatrix[q]);
    printf("],\"energy\":%.17g,\"cfl\":%.17g}", cd.ParticleEnergy, cd.cflCell[0]);
    blk.block->FirstCellParticleTable[ci + NX * (cj + NX * ck)] = -1;
  }
  printf("],");

  // ---- Lapenta2017 on particles of the block interior ----
  PIC::Mover::cLapentaInputData data;
  data.E_Corner = blk.E.data();
  data.B_C = kCenterB ? blk.Bcen.data() : blk.B.data();
  data.MolMass = PIC::MolecularData::MolMass;
  data.ElectricChargeTable = PIC::MolecularData::ElectricChargeTable;
  data.TimeStepTable = PIC::ParticleWeightTimeStep::GlobalTimeStep;
  data.ParticleDataLength = L;
  data.ParticleDataBuffer = buf.data();
  data.mesh = PIC::Mesh::mesh;
  data.node = blk.node;
  printf("\"lapenta\":[");
  for (int n = 0; n < 200; n++) {
    Particle q;
    for (int d = 0; d < 3; d++) q.x[d] = (0.5 + (NX - 1.0) * rng.next()) * dx;
    const int species = n % 2;
    use_species(species);
    q.s = 0;
    const double vt = species ? 0.01 : 0.05;
    for (int d = 0; d < 3; d++) q.v[d] = vt * (2.0 * rng.next() - 1.0) * 1.7;
    q.w = 1.0;
    const long ptr = next_free++;
    PIC::ParticleBuffer::byte* pp = buf.data() + ptr * L;
    put(pp, q, -1, -1);
    const int code = PIC::Mover::Lapenta2017(pp, ptr, &data);
    Particle r = q;
    PIC::ParticleBuffer::GetX(r.x, pp);
    PIC::ParticleBuffer::GetV(r.v, pp);
    int i, j, k;
    PIC::Mesh::mesh->FindCellIndex(r.x, i, j, k, blk.node, false);
    printf("%s{\"species\":%d,\"in\":", n ? "," : "", species);
    print_particle(q);
    printf(",\"x\":[%.17g,%.17g,%.17g],\"v\":[%.17g,%.17g,%.17g],\"code\":%d,\"cell\":[%d,%d,%d]}",
           r.x[0], r.x[1], r.x[2], r.v[0], r.v[1], r.v[2], code, i, j, k);
  }
  printf("],");

  // ---- Boris on particles of the block interior (E = E^{n+theta} slot
  // values, B = corner B: the same corner arrays) ----
  PIC::Mesh::mesh->rootTree = blk.node;
  g_hook_E = blk.E.data();
  g_hook_B = blk.B.data();
  printf("\"boris\":[");
  for (int n = 0; n < 200; n++) {
    Particle q;
    for (int d = 0; d < 3; d++) q.x[d] = (0.5 + (NX - 1.0) * rng.next()) * dx;
    const int species = n % 2;
    use_species(species);
    q.s = 0;
    const double vt = species ? 0.01 : 0.05;
    for (int d = 0; d < 3; d++) q.v[d] = vt * (2.0 * rng.next() - 1.0) * 1.7;
    q.w = 1.0;
    const long ptr = next_free++;
    PIC::ParticleBuffer::byte* pp = buf.data() + ptr * L;
    put(pp, q, -1, -1);
    const int code = PIC::Mover::Boris(ptr, 2.5 * dt, blk.node);
    Particle r = q;
    PIC::ParticleBuffer::GetX(r.x, pp);
    PIC::ParticleBuffer::GetV(r.v, pp);
    int i, j, k;
    PIC::Mesh::mesh->FindCellIndex(r.x, i, j, k, blk.node, false);
    printf("%s{\"species\":%d,\"dt\":%.17g,\"in\":", n ? "," : "", species, 2.5 * dt);
    print_particle(q);
    printf(",\"x\":[%.17g,%.17g,%.17g],\"v\":[%.17g,%.17g,%.17g],\"code\":%d,\"cell\":[%d,%d,%d]}",
           r.x[0], r.x[1], r.x[2], r.v[0], r.v[1], r.v[2], code, i, j, k);
  }
  printf("]}\n");
  return 0;
}
