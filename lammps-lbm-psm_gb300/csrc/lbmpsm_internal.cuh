// lbmpsm_internal.cuh -- shared definitions of the GB300 LBM-PSM library.
//
// Device data layout (one lattice = one handle):
//   populations  SoA, f[q*Np + node], node = (sz*S1 + sy)*P0 + sx, x fastest,
//                rows padded to a pitch P0 that is a multiple of 8.
//                In-place "A-A" streaming: even steps read and write a node's
//                own slots (writing direction q into slot opp(q)), odd steps
//                gather from and scatter to the neighbours.  One copy of the
//                populations, every population read once and written once per
//                step.
//   storage extents S[d]: periodic axes hold only the n interior nodes and
//                wrap; non-periodic axes also hold the two halo planes of the
//                reference lattice (which collides them and whose populations
//                streamed in from outside the array stay at the initial
//                equilibrium w_q).  Reference halo index h = s + off[d].
//   particle table per node (the reference's ParticleDataOnLattice without
//                its force slots): flag (bit0/bit1 = slot occupied), ids,
//                eps, us in FP64, and an FP32 mirror for the FP32/FP16
//                collision kernels.  Node forces of the current step are
//                written per PSM node and reduced per particle image.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lbmpsm {

// ---------------------------------------------------------------- lattices
// Velocity sets and weights of src/LBM_PSM_lattice.h:186-209.
struct D2Q9 {
  static constexpr int Q = 9;
  static constexpr int DIM = 2;
  __host__ __device__ static constexpr int ex(int q) {
    return (q == 1 || q == 5 || q == 8) ? 1 : ((q == 3 || q == 6 || q == 7) ? -1 : 0);
  }
  __host__ __device__ static constexpr int ey(int q) {
    return (q == 2 || q == 5 || q == 6) ? 1 : ((q == 4 || q == 7 || q == 8) ? -1 : 0);
  }
  __host__ __device__ static constexpr int ez(int) { return 0; }
  __host__ __device__ static constexpr int opp(int q) {
    return q == 0 ? 0 : (q <= 4 ? ((q + 1) % 4) + 1 : ((q - 5 + 2) % 4) + 5);
  }
  __host__ __device__ static constexpr double w(int q) {
    return q == 0 ? 4.0 / 9.0 : (q <= 4 ? 1.0 / 9.0 : 1.0 / 36.0);
  }
};

struct D3Q19 {
  static constexpr int Q = 19;
  static constexpr int DIM = 3;
  __host__ __device__ static constexpr int ex(int q) {
    return (q == 1 || q == 7 || q == 9 || q == 13 || q == 15)
               ? 1
               : ((q == 2 || q == 8 || q == 10 || q == 14 || q == 16) ? -1 : 0);
  }
  __host__ __device__ static constexpr int ey(int q) {
    return (q == 3 || q == 7 || q == 11 || q == 14 || q == 17)
               ? 1
               : ((q == 4 || q == 8 || q == 12 || q == 13 || q == 18) ? -1 : 0);
  }
  __host__ __device__ static constexpr int ez(int q) {
    return (q == 5 || q == 9 || q == 11 || q == 16 || q == 18)
               ? 1
               : ((q == 6 || q == 10 || q == 12 || q == 15 || q == 17) ? -1 : 0);
  }
  __host__ __device__ static constexpr int opp(int q) {
    return q == 0 ? 0 : ((q & 1) ? q + 1 : q - 1);
  }
  __host__ __device__ static constexpr double w(int q) {
    return q == 0 ? 1.0 / 3.0 : (q <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
  }
};

// Exact small-integer to float conversion without the conversion unit:
// valid for |k| < 2^22.
__device__ __forceinline__ float small_int_to_float(int k) {
  return __int_as_float(0x4B400000 + k) - 12582912.0f;
}

// Division by a runtime divisor without the conversion unit (integer
// division otherwise goes through int/float conversions, which share the slow
// FP64 pipe on this GPU): q = umulhi(n, ceil(2^32/d)), exact for n*d < 2^32
// (checked exhaustively for d <= 4096, n < 2^22).
struct FastDiv {
  unsigned d, m;
};
__host__ __device__ __forceinline__ FastDiv make_fastdiv(unsigned d) {
  FastDiv f;
  f.d = d;
  f.m = d > 1 ? 0xFFFFFFFFu / d + 1u : 0u;
  return f;
}
__device__ __forceinline__ unsigned fast_div(unsigned n, const FastDiv& f) {
  return f.d > 1 ? __umulhi(n, f.m) : n;
}

// ---------------------------------------------------------------- geometry
struct Geom {
  int dim, Q;
  int L[3];    // reference local sizes including halo (L[2] = 1 in 2-D)
  int S[3];    // device storage extents
  int off[3];  // reference index h = s + off
  int per[3];  // periodic axes wrap; the 2-D z axis counts as periodic
  int P0;      // x pitch: S0 rounded up to 8 so that every x-row starts 16-byte aligned
  long long N; // P0*S1*S2 (node slots including the x padding)
  long long Np;// population stride (N rounded up to 64)
  // A batched ensemble stacks nbox boxes of equal geometry along z: box b
  // holds storage planes [b*bz, (b+1)*bz) and its z axis wraps (or ends)
  // within them.  One lattice is a batch of one box (bz = S[2]).
  int bz, nbox;
  FastDiv fbz;
};

// box of storage plane sz and its plane within the box
__device__ __forceinline__ int box_of_z(const Geom& g, int sz) {
  return g.nbox > 1 ? (int)fast_div((unsigned)sz, g.fbz) : 0;
}

__host__ __device__ __forceinline__ long long node_index(const Geom& g, int sx, int sy, int sz) {
  return ((long long)sz * g.S[1] + sy) * g.P0 + sx;
}

// Neighbour offsets of one node: o[axis][0] towards -1, o[axis][1] towards +1
// (in nodes); v bit (2*axis + side) set when that neighbour exists.
struct Nbr {
  int o[3][2];
  unsigned v;
};

__device__ __forceinline__ Nbr make_nbr(const Geom& g, int sx, int sy, int sz) {
  Nbr nb;
  nb.v = 0;
  const int s[3] = {sx, sy, sz - box_of_z(g, sz) * g.bz};  // z within its box
  const int stride[3] = {1, g.P0, g.P0 * g.S[1]};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int n = a == 2 ? g.bz : g.S[a];
    // towards -1
    if (s[a] > 0) {
      nb.o[a][0] = -stride[a];
      nb.v |= 1u << (2 * a);
    } else if (g.per[a]) {
      nb.o[a][0] = (n - 1) * stride[a];
      nb.v |= 1u << (2 * a);
    } else {
      nb.o[a][0] = 0;
    }
    // towards +1
    if (s[a] < n - 1) {
      nb.o[a][1] = stride[a];
      nb.v |= 1u << (2 * a + 1);
    } else if (g.per[a]) {
      nb.o[a][1] = -(n - 1) * stride[a];
      nb.v |= 1u << (2 * a + 1);
    } else {
      nb.o[a][1] = 0;
    }
  }
  return nb;
}

// offset and existence of the neighbour in direction (cx, cy, cz), c in {-1,0,1}
__device__ __forceinline__ int nbr_off(const Nbr& nb, int cx, int cy, int cz) {
  int o = 0;
  if (cx) o += nb.o[0][cx > 0];
  if (cy) o += nb.o[1][cy > 0];
  if (cz) o += nb.o[2][cz > 0];
  return o;
}
__device__ __forceinline__ bool nbr_ok(const Nbr& nb, int cx, int cy, int cz) {
  bool ok = true;
  if (cx) ok = ok && ((nb.v >> (0 + (cx > 0))) & 1u);
  if (cy) ok = ok && ((nb.v >> (2 + (cy > 0))) & 1u);
  if (cz) ok = ok && ((nb.v >> (4 + (cz > 0))) & 1u);
  return ok;
}

// ---------------------------------------------------------------- particle table
struct Table {
  uint8_t* flag;   // N
  int2* ids;       // N
  double2* eps;    // N (FP64 storage only; null otherwise)
  double* us;      // 6N  (slot-major: us[6n + 3*slot + c]; FP64 storage only)
  float4* rec32;   // 2N  (eps, usx, usy, usz) per slot, FP32 mirror
  void* nodeF;     // 6N  FP64 (FP64 storage) or FP32 (other storages)
};

// ---------------------------------------------------------------- step params
// Parameters that differ between the boxes of a batched ensemble (for one
// lattice: its own parameters).
struct BoxParams {
  double omega, one_minus_omega, guo_pref, tau;  // BGK / Guo, FP64
  double F[3];                                   // F_lbm
  float omega_f, omo_f, gpref_f, tm_f;           // FP32 copies made on the host
  float F_f[3];
  int has_force;                                 // |F_lbm|^2 > 0
  double origin[3];                              // the box's own frame
  double Uc, u_lb, tc, dt_d;                     // UnitConversion
  double forceFactor, torqueFactor;
};

// launch shape of the row-pipelined FP32/FP16 collide kernel (grid 0: the
// direct kernel instead)
struct PipeConfig {
  int grid = 0, threads = 0, stages = 0;
  size_t smem = 0;
  int dy = 0, dz = 0;  // grid = dz * S1 + dy
};

struct CollideParams {
  Geom g;
  void* f;                // populations (double / float / half)
  Table tab;
  double* rho_out;        // optional macro output (N), FP64
  double* u_out;          // optional (3N)
  int store_macro;
  int weighting;          // LBMPSM_WEIGHT_*
  const BoxParams* box;   // per-box BGK / Guo parameters (g.nbox entries)
  int has_force;          // any box with |F_lbm|^2 > 0
  double invCs2, invCs4;
  float scale16;          // FP16 storage: stored value = deviation * scale16 (= 2^FP16_SCALE_LOG2)
  int* status;            // error word (STATUS_*)
  PipeConfig pipe;
  const void* fsrc;       // FP64 only: read the populations here and write f (null: in place)
  long long full_wait_limit;  // polls of the row pipeline's consumers on a stage's arrival
                              // before they give up (STATUS_TIMEOUT): 0 = the default limit,
                              // < 0 = none at all (give up at once; a test of the timeout path)
};


// One collide launch over several lattices (the members of a group, e.g. one
// batched ensemble per box size): the blocks take tiles of one member each.
// The row pipeline (FP32 / FP16 / BF16) packs k consecutive x-rows of a
// storage plane into a tile, so that small boxes fill the block's threads;
// the FP64 kernel takes the members' (row, x-chunk) blocks in turn.  Members
// must be 3-D and periodic on every axis.
// FP16 storage keeps deviations scaled by 2^12; the collide kernels work on
// the scaled values directly (a power-of-two scale commutes with rounding).
constexpr int FP16_SCALE_LOG2 = 12;
constexpr int MULTI_MAX = 16;
struct MultiMember {
  CollideParams p;  // the member's own collide parameters
  int k;            // rows per tile (row pipeline)
  int tpp;          // tiles per storage plane, ceil(S1 / k)
  FastDiv ftpp;     // division by tpp
  int has_force;    // the member has a body force (Guo terms)
};
struct MultiCollide {
  const MultiMember* m;       // nm entries in device memory
  int nm;
  int first[MULTI_MAX + 1];   // first tile (row pipeline) or block (FP64) of each member;
                              // first[nm] = total
  int tcp;                    // row pipeline: stage capacity per direction (elements)
  PipeConfig pipe;            // row pipeline: grid, threads, shared memory, stages
  int any_force;
  int* status;
  long long full_wait_limit;  // as CollideParams
};

// Zou-He face list of one `fix lbm-psm-bc` keyword.
enum FaceKind {
  FACE_VEL2_XN, FACE_VEL2_XP, FACE_DENS2_XP, FACE_VEL2_YN, FACE_VEL2_YP,
  FACE_VEL3_XN, FACE_VEL3_XP, FACE_DENS3_XP, FACE_VEL3_YN, FACE_VEL3_YP,
  FACE_VEL3_ZN, FACE_VEL3_ZP
};
struct Face {
  int kind;
  int axis;        // normal axis
  int plane;       // storage index of the face plane along axis
  int lo[3], hi[3];// inclusive storage ranges of the face nodes (axis: plane..plane)
  double p0;       // velocity (vel faces) or density (dens faces)
};
struct BCParams {
  Geom g;
  void* f;
  int nfaces;
  Face face[6];
  int after_odd;   // 1: the last step was odd (natural layout), 0: even (swapped layout)
  float scale16;
};

// ---------------------------------------------------------------- particles
struct Img {
  int tag;
  int valid;          // box non-empty on the device lattice
  int lo[3], hi[3];   // map box, storage coordinates, [lo, hi)
  int clo[3], chi[3]; // cell range touched, inclusive
  double xl[3];       // lattice-local centre (reference halo frame)
  double r;           // radius, lattice units
  double uT[3];       // translational velocity, lattice units
  double om[3];       // angular velocity, lattice units
  // exact FP64 thresholds of calcSolidFraction (r+h)^2, (r-h)^2, r^2
  double rP2, rM2, rSq;
  // FP32 helpers: xl = xi + xfrac exactly; node offset dx = (h - xi) - xfrac
  int xi[3];
  float xf[3];
  float rP2f, rM2f, rSqf;
  int has_spin;       // any omega component non-zero
  long long sf_off;   // offset of this image's box in the solid-fraction code scratch
  int box[3];         // box extents (hi - lo)
  int rlo[3], rhi[3]; // force-reduction box, reference frame, clamped to interior nodes
  float uTf[3], omf[3];  // FP32 roundings of uT and om (FP32 / FP16 storage)
  int solo;           // no periodic copy of the particle can have an overlapping box
  int qlo[3], qhi[3]; // part of the reduction box the reduction visits
  int bidx;           // box of a batched ensemble (0 for one lattice)
  int zoff;           // its first storage plane (bidx * bz); lo/hi above are global
};

// Solid-fraction codes of one (image, node) pair: 0..1000 = number of
// sub-cell centres inside (sf = n/10^d), SF_ONE = the early-out value 1.0.
constexpr unsigned short SF_ONE = 0xFFFF;

struct MapParams {
  Geom g;
  Table tab;
  int n;
  const int* tag;
  const double* x;
  const double* v;
  const double* omega;
  const double* radius;
  const int* img_box;  // box of each image (batched ensemble) or null (all box 0)
  const BoxParams* box;
  double dx;
  double sqrt2half;   // sqrt(2.1)/2 in 2-D, sqrt(3.1)/2 in 3-D (host libm)
  Img* img;
  // optional copies of the image arrays (tag; x | v | omega | radius), written
  // by img_prep when it reads a caller's arrays in place
  int* copy_tag;
  double* copy_xvw;
  // per image, three int4 for the table update: (lo0 | hi0 << 16, lo1 | hi1 << 16,
  // lo2 | hi2 << 16, tag), (sf_off low, sf_off high, box0 | box1 << 16, has_spin),
  // (uTf[0..2] as bits, 0); an image with an empty box has lo = hi = 0
  int4* arec;
  int cb[3];          // cell edge (nodes) per axis
  int C[3];           // cells per axis
  int* cell_count;
  int* cell_off;
  int* cell_fill;
  int* list;
  int4* lrec;         // per cell-list entry: its image's three records above (the
                      // third with the image index in w), written by cell_sort
  long long list_cap;
  unsigned long long* pair_total;  // [0] cell-list pairs, [1] solid-fraction codes, [2] shell nodes
  unsigned short* sfcode;          // codes of all (image, box node) pairs
  long long sf_cap;
  const double* sf_value;          // sf_value[n] = n/10^d (n = 0..1000), FP64
  const float* sf_value32;         // its FP32 roundings
  int4* shell;                     // shell nodes: image, box index, x | y << 16, z
  long long shell_cap;
  int sm_count;                    // multiprocessors (persistent grids)
  int* status;
  int write32;        // also write the FP32 mirror
};

struct ReduceParams {
  Geom g;
  Table tab;
  const Img* img;     // image records of the step's map (centre, box)
  const BoxParams* box;
  int n;
  const int* tag;
  int nodeF_is_double;
  double* fh;
  double* th;
  double* S;
  double* fh2;        // optional second copies of the outputs (the caller's
  double* th2;        // buffers of lbmpsm_step_device or, read over NVLink-C2C,
  double* S2;         // of lbmpsm_step), written with the first
  const int* status;  // the step's status word (device)
  int* status_out;    // optional host-visible copy of it, written by block 0 last
};

// status bits
enum : int { STATUS_LIST_OVERFLOW = 1, STATUS_NONFINITE = 2, STATUS_TIMEOUT = 4,
             STATUS_ADJ_CROWDED = 8, STATUS_ADJ_SAME_TAG = 16 };

// ---------------------------------------------------------------- adjoint
// Dense per-node data of the adjoint and tangent sweeps (N entries each).
// An "entry" is a table slot: the table's particle when the slot is taken,
// else the particle that would take it if its solid fraction rose above
// zero (one whose surface shell holds the node).
struct AdjNodes {
  uint8_t* band;   // node in the surface shell of some particle image
  int2* tag;       // entry tag per slot (0: none)
  double* us;      // 6N, slot-major: solid velocity of entering particles
  int2* cw;        // images of the entry's tag whose reduction box holds the node
  double* sigma;   // 2N: sum over steps of dJ/dB per slot (band nodes)
  double* edot;    // 2N: tangent solid-fraction rate per slot
};

struct AdjParams {
  Geom g;
  Table tab;
  BoxParams bp;
  int weighting;
  AdjNodes an;
  const double* state;  // A-A populations before the step (FP64)
  int odd;              // A-A parity of that state
  const double* lin;    // adjoint: lambda of the next step; tangent: this step's tangent
  double* lout;         // adjoint: lambda of this step; tangent: the next step's tangent
  double c;             // objective weight of this step
  double d[3];          // drag direction
  double* part;         // per-block partial sums, ADJ_PART per block
  double domega, dtau, dF[3];  // tangent direction (lattice units)
};
constexpr int ADJ_PART = 5;  // d/domega, d/dtau through B, d/dF[3] (tangent: dJ in [0])

struct AdjSetup {
  Geom g;
  Table tab;
  AdjNodes an;
  const Img* img;
  int n;
  const int* cell_off;
  const int* cell_count;
  const int* list;
  int cb[3], C[3];
  double h0;    // early-out half-diagonal of calcSolidFraction
  double hl;    // centre step, lattice units
  int* status;
};

struct AdjCentre {
  Geom g;
  Table tab;
  AdjNodes an;
  const Img* img;
  int n;
  const double* x;      // physical image centres (3n)
  double origin[3], dx;
  double h;             // centre step, physical units
  double h0;
  double tau;
  int weighting;
  const double* xdot;   // tangent: centre direction per image (3n); null for the adjoint
  double* out;          // adjoint: dJ/dx per image (3n)
};

// ---------------------------------------------------------------- launchers
// collide.cu / collide_f32.cu
cudaError_t launch_collide_f64(const CollideParams& p, int odd, cudaStream_t st);
cudaError_t launch_collide_f32(const CollideParams& p, int odd, cudaStream_t st);
cudaError_t launch_collide_f16(const CollideParams& p, int odd, cudaStream_t st);
cudaError_t launch_collide_bf16(const CollideParams& p, int odd, cudaStream_t st);
// storage 1 (FP32), 2 (FP16) or 3 (BF16); sets the kernels' shared-memory limit and
// sizes the persistent grid from the occupancy on this device (stages 0:
// the direct kernel, cfg left empty)
cudaError_t prepare_collide_lowp(const Geom& g, int storage, int sm_count, int stages,
                                 PipeConfig* cfg);
// times the candidate launch shapes (pipeline stages 3, 2, 4, 5) on p.f and
// stores the fastest in best (unchanged if none fits), the per-pair times in
// ms_out (-1: shape does not fit)
constexpr int LBMPSM_TUNE_CANDIDATES = 4;
cudaError_t tune_collide_lowp(CollideParams p, int storage, int sm_count, cudaStream_t st,
                              PipeConfig* best, float* ms_out);
// one launch over the members of mc (storage 0: FP64, 1: FP32, 2: FP16, 3: BF16);
// prepare_collide_multi fills mc.first, tcp, pipe and the members' k / tpp
// from their geometries (host copies in members) and the device's occupancy
cudaError_t prepare_collide_multi(MultiCollide& mc, MultiMember* members, int storage, int sm_count);
cudaError_t launch_collide_multi(const MultiCollide& mc, int storage, int odd, cudaStream_t st);
cudaError_t launch_collide_f64_multi(const MultiCollide& mc, int odd, cudaStream_t st);
cudaError_t launch_bc_f64(const BCParams& p, cudaStream_t st);
cudaError_t launch_bc_f32(const BCParams& p, cudaStream_t st);
cudaError_t launch_bc_f16(const BCParams& p, cudaStream_t st);
cudaError_t launch_bc_bf16(const BCParams& p, cudaStream_t st);
// population layout conversions (storage <-> reference AoS with halo, FP64)
cudaError_t launch_init_populations(const Geom& g, void* f, int storage, float scale16,
                                    cudaStream_t st);
cudaError_t launch_get_populations(const Geom& g, const void* f, int storage, int after_odd,
                                   float scale16, double* out_ref, cudaStream_t st);
cudaError_t launch_set_populations(const Geom& g, void* f, int storage, int after_odd,
                                   float scale16, const double* in_ref, cudaStream_t st);
cudaError_t launch_check(const Geom& g, const void* f, int storage, int after_odd,
                         float scale16, double* acc4, int* status, cudaStream_t st);
// particles.cu
// aux, fork and join (may all be null: one stream) let the cell-list kernels
// run beside the solid-fraction kernels
cudaError_t launch_map(const MapParams& p, cudaStream_t st, cudaStream_t aux = nullptr,
                       cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr);
cudaError_t launch_reduce(const ReduceParams& p, cudaStream_t st);
// the kernels whose arguments a replayed device-step graph updates per call
const void* img_prep_fn();
const void* reduce_fn(int nodeF_is_double);
cudaError_t launch_table_export(const Geom& g, const Table& t, int* ids, double* eps,
                                double* us, cudaStream_t st);
cudaError_t launch_export_fields(const Geom& g, const Table& t, const double* rho,
                                 const double* u, int as_double, double B0, double rho0,
                                 double u0, void* solid_out, void* rho_out, void* u_out,
                                 cudaStream_t st);
// adjoint.cu
long long adj_blocks(const Geom& g);
cudaError_t launch_adj_entries(const AdjSetup& s, cudaStream_t st);
cudaError_t launch_adj_step(const AdjParams& p, int tangent, cudaStream_t st);
cudaError_t launch_adj_centre(const AdjCentre& c, cudaStream_t st);
cudaError_t launch_adj_drag(const double* fh, int n, double d0, double d1, double d2,
                            double* out, cudaStream_t st);
cudaError_t launch_adj_sum(const double* part, long long nblocks, double* out, cudaStream_t st);

}  // namespace lbmpsm
