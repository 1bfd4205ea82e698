// particles.cu -- particle <-> lattice kernels (FP64, compiled with -fmad=false).
//
// Map (replaces ExchangeParticleData::setParticlesOnLattice and
// calcSolidFraction, src/LBM_PSM_exchangeParticleData.cpp:24-169, with
// LBMPSMLattice::setParticleOnLattice / setToZero,
// src/LBM_PSM_lattice.cpp:257-324).  The reference walks the particle images
// in array order and, for each, the nodes of its bounding box, updating a
// persistent two-slot table per node; the final table depends on that order.
// Here every node applies, in its own thread, the updates of the images whose
// boxes contain it in ascending image order, which yields the same table
// without atomics on the table:
//   1. img_prep   : per image, box in device coordinates, coarse cells touched
//   2. cell_scan  : offsets of the per-cell image lists
//   3. img_fill   : scatter image ids into the cell lists
//   4. cell_sort  : sort each list ascending (restores image order)
//   5. node_apply : per node, walk its cell's list and apply the 4-way update
// The solid fraction counts the reference's 10^d sub-cell centres; each
// comparison is decided in FP32 when it is far from the threshold (a margin
// 250x the worst FP32 error) and otherwise evaluated with the reference's
// FP64 expression, so the count is the reference's count.
//
// Reduce (replaces calculateHydrodynamicInteractions,
// src/LBM_PSM_exchangeParticleData.cpp:172-244): one block per image sums
// the node forces of its tag over the box clamped to interior nodes, with a
// fixed-order warp-shuffle and block reduction (deterministic run to run).
#include "lbmpsm_internal.cuh"

namespace lbmpsm {

static __device__ __forceinline__ int clampi(int v, int lo, int hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

// lattice-local centre on one rank (src/LBM_PSM_exchangeParticleData.cpp:31-37)
static __device__ __forceinline__ double local_centre(double x, double origin, double dx) {
  const double g = (x - origin) / dx;
  return g - ((0 - ((double)0 * 2.0 * (double)1)) - 1);
}

// Box of one image for the force reduction, clamped to interior nodes
// (src/LBM_PSM_exchangeParticleData.cpp:188-195).
static __device__ __forceinline__ void reduce_box_of(const Geom& g, const double xl[3], double r,
                                                     int lo[3], int hi[3]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int a = (int)(xl[d] - r) - 2;
    int c = (int)(xl[d] + r) + 2;
    if (d < 2 || g.dim == 3) {
      a = clampi(a, 1, g.L[d] - 1);
      c = clampi(c, 1, g.L[d] - 1);
      if (d == 2) {
        if (a < 0) a = 0;
        if (c < 1) c = 1;
      }
    } else {
      // fmax(fmin(fmax(z, 1), nz - 1), slot) with nz = 1 in 2-D
      a = a < 1 ? 1 : a;
      a = a > g.L[2] - 1 ? g.L[2] - 1 : a;
      a = a < 0 ? 0 : a;
      c = c < 1 ? 1 : c;
      c = c > g.L[2] - 1 ? g.L[2] - 1 : c;
      c = c < 1 ? 1 : c;
    }
    lo[d] = a;
    hi[d] = c;
  }
}

// One thread per image builds its record (the FP64 arithmetic of
// src/LBM_PSM_exchangeParticleData.cpp:31-55), counts the image into the
// cells its box touches, and the warp reserves its images' ranges of
// solid-fraction codes with one atomic.
// Images per block of img_prep (a partial warp): each thread's image record
// is a long FP64 chain, and FP64 runs at 1/64 of the FP32 rate on this GPU,
// so the images are spread over as many multiprocessors as possible.
constexpr int IMG_LANES = 16;
__global__ void img_prep_kernel(MapParams p) {
  constexpr unsigned M = IMG_LANES == 32 ? 0xffffffffu : (1u << IMG_LANES) - 1u;
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool mine = i < p.n;
  int cr[6] = {0, 0, 0, -1, -1, -1};  // clo[3], chi[3]
  unsigned long long vol = 0;
  Img im;
  if (mine) {
    const Geom& g = p.g;
    im.tag = p.tag[i];
    if (p.copy_tag) {  // the caller's arrays, kept for later steps with these images
      const size_t nn = (size_t)p.n;
      p.copy_tag[i] = im.tag;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        p.copy_xvw[3 * (size_t)i + c] = p.x[3 * (size_t)i + c];
        p.copy_xvw[3 * nn + 3 * (size_t)i + c] = p.v[3 * (size_t)i + c];
        p.copy_xvw[6 * nn + 3 * (size_t)i + c] = p.omega[3 * (size_t)i + c];
      }
      p.copy_xvw[9 * nn + i] = p.radius[i];
    }
    im.bidx = p.img_box ? p.img_box[i] : 0;
    im.zoff = im.bidx * g.bz;
    const BoxParams& bp = p.box[im.bidx];
    const double r = p.radius[i] / p.dx;
    im.r = r;
    bool valid = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double xl = local_centre(p.x[3 * i + d], bp.origin[d], p.dx);
      im.xl[d] = xl;
      int lo = (int)(xl - r) - 2;
      int hi = (int)(xl + r) + 2;
      lo = clampi(lo, 0, g.L[d]);
      hi = clampi(hi, 0, g.L[d]);
      if (d == 2) {  // 2-D keeps its single z layer
        if (lo < 0) lo = 0;
        if (hi < 1) hi = 1;
      }
      // reference halo frame -> device storage
      int slo, shi;
      if (g.off[d] == 1) {
        slo = (lo < 1 ? 1 : lo) - 1;
        shi = (hi > g.L[d] - 1 ? g.L[d] - 1 : hi) - 1;
      } else {
        slo = lo;
        shi = hi;
      }
      const int z0 = d == 2 ? im.zoff : 0;  // boxes of an ensemble stack along z
      im.lo[d] = slo + z0;
      im.hi[d] = shi + z0;
      if (slo >= shi) valid = false;
      im.uT[d] = p.v[3 * i + d] / bp.Uc * bp.u_lb;
      im.om[d] = p.omega[3 * i + d] * bp.tc * bp.dt_d;
      im.uTf[d] = (float)im.uT[d];
      im.omf[d] = (float)im.om[d];
    }
    im.valid = valid;
    const double rP = r + p.sqrt2half;
    const double rM = r - p.sqrt2half;
    im.rP2 = rP * rP;
    im.rM2 = rM * rM;
    im.rSq = r * r;
    im.rP2f = (float)im.rP2;
    im.rM2f = (float)im.rM2;
    im.rSqf = (float)im.rSq;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      // xl = xi + xfrac exactly (the fractional part of a double is exact)
      const double xl = im.xl[d];
      const bool small = fabs(xl) < 1.0e9;
      const double fl = small ? floor(xl) : 0.0;
      im.xi[d] = (int)fl;
      im.xf[d] = (float)(xl - fl);
    }
    // the node velocity reduces to uT + 0.0 bit for bit when every omega
    // component is +0.0 and no uT component is -0.0 (signed-zero arithmetic)
    bool plain = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (__double_as_longlong(im.om[d]) != 0ll) plain = false;
      if (__double_as_longlong(im.uT[d]) == (long long)0x8000000000000000ull) plain = false;
    }
    im.has_spin = plain ? 0 : 1;
    reduce_box_of(g, im.xl, r, im.rlo, im.rhi);
    // When no periodic copy of this particle can have an overlapping box
    // (box width below the period on every periodic axis), the nodes of the
    // box that hold its tag after the map all have eps > 0 from this image,
    // hence lie within the early-out radius rP: the reduction then only
    // visits the box part around the sphere (and still checks each tag).
    {
      bool solo = true;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if (d >= g.dim) break;
        const int w = ((int)(im.xl[d] + r) + 2) - ((int)(im.xl[d] - r) - 2);
        if (g.per[d] && w >= (d == 2 ? g.bz : g.S[d])) solo = false;
      }
      im.solo = solo ? 1 : 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        im.qlo[d] = im.rlo[d];
        im.qhi[d] = im.rhi[d];
        if (solo && (d < 2 || g.dim == 3)) {
          const int a = (int)floor(im.xl[d] - rP), b = (int)floor(im.xl[d] + rP) + 1;
          im.qlo[d] = max(im.qlo[d], a);
          im.qhi[d] = min(im.qhi[d], b);
        }
      }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) im.box[d] = valid ? im.hi[d] - im.lo[d] : 0;
    if (valid) {
      vol = (unsigned long long)im.box[0] * im.box[1] * im.box[2];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        im.clo[d] = im.lo[d] / p.cb[d];
        im.chi[d] = (im.hi[d] - 1) / p.cb[d];
        cr[d] = im.clo[d];
        cr[3 + d] = im.chi[d];
      }
    } else {
#pragma unroll
      for (int d = 0; d < 3; ++d) im.clo[d] = 0, im.chi[d] = -1;
    }
  }
  // code ranges: warp prefix of the box volumes, one atomic per warp
  unsigned long long incl = vol;
#pragma unroll
  for (int o = 1; o < IMG_LANES; o <<= 1) {
    const unsigned long long x = __shfl_up_sync(M, incl, o);
    if (lane >= o) incl += x;
  }
  unsigned long long base = 0;
  if (lane == IMG_LANES - 1) base = atomicAdd(&p.pair_total[1], incl);
  base = __shfl_sync(M, base, IMG_LANES - 1);
  if (mine) {
    im.sf_off = (long long)(base + incl - vol);
    p.img[i] = im;
    int4 a = make_int4(0, 0, 0, im.tag), b;
    if (im.valid)
      a = make_int4(im.lo[0] | (im.hi[0] << 16), im.lo[1] | (im.hi[1] << 16),
                    im.lo[2] | (im.hi[2] << 16), im.tag);
    b = make_int4((int)(unsigned)(unsigned long long)im.sf_off,
                  (int)(unsigned)((unsigned long long)im.sf_off >> 32),
                  im.box[0] | (im.box[1] << 16), im.has_spin);
    p.arec[3 * i] = a;
    p.arec[3 * i + 1] = b;
    p.arec[3 * i + 2] = make_int4(__float_as_int(im.uTf[0]), __float_as_int(im.uTf[1]),
                                  __float_as_int(im.uTf[2]), 0);
  }
  // cell counts: each lane walks the cells its image's box touches (integer
  // sums, so the order of the atomics does not matter); one atomic per warp
  // for the pair total
  unsigned long long pairs = 0;
  if (cr[3] >= cr[0] && cr[4] >= cr[1] && cr[5] >= cr[2]) {
    for (int cz = cr[2]; cz <= cr[5]; ++cz)
      for (int cy = cr[1]; cy <= cr[4]; ++cy) {
        int* row = p.cell_count + (cz * p.C[1] + cy) * p.C[0];
        for (int cx = cr[0]; cx <= cr[3]; ++cx) atomicAdd(row + cx, 1);
      }
    pairs = (unsigned long long)(cr[3] - cr[0] + 1) * (unsigned long long)(cr[4] - cr[1] + 1) *
            (unsigned long long)(cr[5] - cr[2] + 1);
  }
#pragma unroll
  for (int o = IMG_LANES / 2; o > 0; o >>= 1) pairs += __shfl_xor_sync(M, pairs, o);
  if (lane == 0 && pairs) atomicAdd(&p.pair_total[0], pairs);
}

// Exclusive scan of the cell counts: one block of 1024 threads walking tiles
// of 8192 counts (8 consecutive per thread, two 16-byte loads), warp shuffles
// within a tile and a running carry between tiles; the offsets go through
// shared memory so that the stores to global memory are coalesced.
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_PER_THREAD = 8;
__global__ void __launch_bounds__(SCAN_THREADS) cell_scan_kernel(const int* __restrict__ count,
                                                                 int* __restrict__ off,
                                                                 int ncells) {
  constexpr int V = SCAN_PER_THREAD;
  constexpr int TILE = V * SCAN_THREADS;
  __shared__ int wsum[SCAN_THREADS / 32];
  __shared__ int carry_s;
  __shared__ int tile[TILE + TILE / 32];  // one pad word per 32: conflict-free strided writes
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t == 0) carry_s = 0;
  __syncthreads();
  for (int base = 0; base < ncells; base += TILE) {
    const int i0 = base + V * t;
    int v[V];
    if (i0 + V <= ncells) {  // i0 is a multiple of 8: aligned 16-byte loads
      const int4* c4 = reinterpret_cast<const int4*>(count + i0);
#pragma unroll
      for (int k = 0; k < V / 4; ++k) {
        const int4 w = c4[k];
        v[4 * k] = w.x;
        v[4 * k + 1] = w.y;
        v[4 * k + 2] = w.z;
        v[4 * k + 3] = w.w;
      }
    } else {
#pragma unroll
      for (int k = 0; k < V; ++k) v[k] = i0 + k < ncells ? count[i0 + k] : 0;
    }
    int own = 0;
#pragma unroll
    for (int k = 0; k < V; ++k) own += v[k];
    int incl = own;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int x = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += x;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      int w = wsum[lane];
      int wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(0xffffffffu, wi, o);
        if (lane >= o) wi += x;
      }
      wsum[lane] = wi - w;  // exclusive prefix of the warps
    }
    __syncthreads();
    int run = carry_s + wsum[warp] + incl - own;
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const int j = V * t + k;
      tile[j + (j >> 5)] = run;
      run += v[k];
    }
    __syncthreads();
    if (t == SCAN_THREADS - 1) carry_s = run;
    const int m = min(TILE, ncells - base);
    for (int j = t; j < m; j += SCAN_THREADS) off[base + j] = tile[j + (j >> 5)];
    __syncthreads();
  }
}

// One warp per image: the lanes enter the image into its cells' lists.
__global__ void img_fill_kernel(MapParams p) {
  const int lane = threadIdx.x & 31;
  const int i = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (i >= p.n) return;
  if (p.pair_total[0] > (unsigned long long)p.list_cap ||
      p.pair_total[1] > (unsigned long long)p.sf_cap) {
    if (i == 0 && lane == 0) atomicOr(p.status, STATUS_LIST_OVERFLOW);
    return;
  }
  const Img& im = p.img[i];
  if (!im.valid) return;
  const int nx = im.chi[0] - im.clo[0] + 1, ny = im.chi[1] - im.clo[1] + 1,
            nz = im.chi[2] - im.clo[2] + 1;
  const int ncell = nx * ny * nz;
  for (int t = lane; t < ncell; t += 32) {
    const int cx = im.clo[0] + t % nx, cy = im.clo[1] + (t / nx) % ny, cz = im.clo[2] + t / (nx * ny);
    const int c = (cz * p.C[1] + cy) * p.C[0] + cx;
    const int pos = atomicAdd(&p.cell_fill[c], 1);
    p.list[(long long)p.cell_off[c] + pos] = i;
  }
}

__global__ void cell_sort_kernel(MapParams p, int ncells) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  if (p.pair_total[0] > (unsigned long long)p.list_cap) return;
  const int off = p.cell_off[c];
  int* a = p.list + off;
  const int m = p.cell_count[c];
  for (int k = 1; k < m; ++k) {
    const int v = a[k];
    int j = k - 1;
    while (j >= 0 && a[j] > v) {
      a[j + 1] = a[j];
      --j;
    }
    a[j + 1] = v;
  }
  // the images' table-update records in list order (FP32 / FP16 storage)
  if (p.write32)
    for (int k = 0; k < m; ++k) {
      const int ii = a[k];
      int4* r = p.lrec + 3 * ((long long)off + k);
      r[0] = p.arec[3 * ii];
      r[1] = p.arec[3 * ii + 1];
      const int4 u = p.arec[3 * ii + 2];
      r[2] = make_int4(u.x, u.y, u.z, ii);
    }
}

// Early-out part of calcSolidFraction for one node, decided in FP32 with a
// proven margin, else in FP64 with the reference's expressions.  Returns a
// code (0 or SF_ONE) or -1 for a shell node whose sub-cells must be counted.
//
// Offsets dx = (double)h - xl are formed as (h - xi) - xfrac with xl = xi + xfrac
// split exactly, so |dxf - dx| <= u(|dx| + 1), u = 2^-24, and the FP32 squared
// distance obeys |d32 - dist| <= u(5 dist + 2 sum|d|).  The margin m is 16x that.
static __device__ __forceinline__ int classify_node(int hi, int hj, int hk, const Img& im,
                                                    float& dxf, float& dyf, float& dzf) {
  const float u = 5.9604644775390625e-08f;  // 2^-24
  dxf = small_int_to_float(hi - im.xi[0]) - im.xf[0];
  dyf = small_int_to_float(hj - im.xi[1]) - im.xf[1];
  dzf = small_int_to_float(hk - im.xi[2]) - im.xf[2];
  const float d32 = dxf * dxf + dyf * dyf + dzf * dzf;
  const float ad = fabsf(dxf) + fabsf(dyf) + fabsf(dzf);
  const float m = 16.0f * u * (5.0f * d32 + 2.0f * ad + 1.0f + im.rP2f);
  if (d32 > im.rP2f + m) return 0;
  const bool nearP = d32 >= im.rP2f - m;
  const bool nearM = d32 >= im.rM2f - m && d32 <= im.rM2f + m;
  if (nearP || nearM) {
    const double dx = (double)hi - im.xl[0];
    const double dy = (double)hj - im.xl[1];
    const double dz = (double)hk - im.xl[2];
    const double dist = dx * dx + dy * dy + dz * dz;
    if (dist > im.rP2) return 0;
    if (dist < im.rM2) return SF_ONE;
    return -1;
  }
  if (d32 < im.rM2f) return SF_ONE;  // below rM^2 - m: inside for certain
  return -1;
}

// A shell node (between the early-out radii) whose sub-cells all lie on one
// side of the surface: the count calcSolidFraction's loop would give
// (src/LBM_PSM_exchangeParticleData.cpp:151-165), 10^dim or 0, else -1.
// Every FP64 sub-cell sum (dx_sq[i] + dy_sq[j]) + dz_sq[k] is monotone in
// each term and each term is convex in the sub-cell offset, so the largest
// sum is the far corner's (|d| + 0.45 per axis) and the smallest is at least
// the sum of max(|d| - 0.45, 0)^2.  Decided in FP32 with the margin M that
// bounds the FP32 error of every sub-cell sum of the node (the one the shell
// count uses); undecided nodes stay in the shell.
static __device__ __forceinline__ int corner_count(int dim, float dxf, float dyf, float dzf,
                                                   float rSqf) {
  const float u = 5.9604644775390625e-08f;  // 2^-24
  const float ax = fabsf(dxf), ay = fabsf(dyf), az = dim == 3 ? fabsf(dzf) : 0.0f;
  const float Ea = ax + 2.0f, Eb = ay + 2.0f, Ec = az + 2.0f;
  const float M = 16.0f * u * (Ea * Ea + Eb * Eb + (dim == 3 ? Ec * Ec : 0.0f) + rSqf);
  const float fx = ax + 0.45f, fy = ay + 0.45f, fz = az + 0.45f;
  const float far = fx * fx + fy * fy + (dim == 3 ? fz * fz : 0.0f);
  if (far < rSqf - M) return dim == 3 ? 1000 : 100;
  const float nx = fmaxf(ax - 0.45f, 0.0f), ny = fmaxf(ay - 0.45f, 0.0f),
              nz = fmaxf(az - 0.45f, 0.0f);
  const float near = nx * nx + ny * ny + (dim == 3 ? nz * nz : 0.0f);
  if (near > rSqf + M) return 0;
  return -1;
}

constexpr int SFC_THREADS = 64;   // classification: one block per image
constexpr int SFS_THREADS = 128;  // shell counting: persistent warps
constexpr int SFS_BUF = 352;      // per-warp buffer of crossing rows (>= 32 + 32*10)

static __device__ __forceinline__ float sub_offset(int k) {
  return -0.45f + 0.1f * small_int_to_float(k);  // within 1.7u of the reference's delta_k
}

// Phase 1 of the map, one block per image.  The box's codes are first set
// to 0 with coalesced stores; then only the nodes of each x-row that may
// lie within rP (an FP32 bound widened by 0.01 node: a superset of the
// nodes classify_node does not put beyond rP for certain) are classified by
// the early-out radii of calcSolidFraction.  Inside nodes get their code
// here, and so do shell nodes whose sub-cells all lie on one side of the
// surface; the other shell nodes (whose sub-cells must be counted) are
// queued per warp in shared memory and appended to a global list with one
// atomic per flush.  Each warp takes 32 rows at a time, one per lane, and
// walks the nodes of their segments 32 at a time (consecutive lanes on
// consecutive nodes of a row).
constexpr int SFC_QW = 256;  // per-warp queue of shell nodes
__global__ void __launch_bounds__(SFC_THREADS) sf_classify_kernel(MapParams p) {
  const Img& im = p.img[blockIdx.x];
  if (!im.valid) return;
  if (p.pair_total[0] > (unsigned long long)p.list_cap ||
      p.pair_total[1] > (unsigned long long)p.sf_cap)
    return;
  constexpr int NW = SFC_THREADS / 32;
  __shared__ int4 q[NW][SFC_QW];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Geom& g = p.g;
  const int wx = im.box[0], wy = im.box[1], wz = im.box[2];
  const int vol = wx * wy * wz;
  unsigned short* code = p.sfcode + im.sf_off;
  for (int li = threadIdx.x; li < vol; li += SFC_THREADS) code[li] = 0;
  __syncthreads();  // the zeros land before any code of this block
  // reference-frame coordinates of the box's first node
  const int h0 = im.lo[0] + g.off[0], h1 = im.lo[1] + g.off[1];
  const int h2 = im.lo[2] - im.zoff + g.off[2];  // z in the box's own frame
  const float rem0 = im.rP2f * 1.0001f + 0.01f;
  const FastDiv fy = make_fastdiv((unsigned)wy);
  int qn = 0;  // entries in this warp's queue (warp-uniform)
  auto flush = [&]() {
    unsigned long long qb = 0;
    if (lane == 0) qb = atomicAdd(&p.pair_total[2], (unsigned long long)qn);
    qb = __shfl_sync(0xffffffffu, qb, 0);
    for (int k = lane; k < qn; k += 32) {
      const unsigned long long pos = qb + k;
      if (pos < (unsigned long long)p.shell_cap)
        p.shell[pos] = q[warp][k];
      else
        atomicOr(p.status, STATUS_LIST_OVERFLOW);
    }
    __syncwarp();
    qn = 0;
  };
  const int R = wy * wz;
  for (int r0 = warp * 32; r0 < R; r0 += SFC_THREADS) {
    const int r = r0 + lane;
    int xa = 0, len = 0, by = 0, bz = 0;
    if (r < R) {
      bz = (int)fast_div((unsigned)r, fy);
      by = r - bz * wy;
      const float dy = small_int_to_float(h1 + by - im.xi[1]) - im.xf[1];
      const float dz = small_int_to_float(h2 + bz - im.xi[2]) - im.xf[2];
      const float rem = rem0 - dy * dy - dz * dz;
      if (rem >= 0.0f) {
        const float h = sqrtf(rem) + 0.01f;
        xa = max(0, im.xi[0] + (int)ceilf(im.xf[0] - h) - h0);
        const int xb = min(wx, im.xi[0] + (int)floorf(im.xf[0] + h) + 1 - h0);
        len = max(xb - xa, 0);
      }
    }
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const int excl = incl - len;
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    for (int base = 0; base < total; base += 32) {
      const int t = base + lane;
      // the row holding node t: the last lane whose offset is <= t
      int l = 0;
#pragma unroll
      for (int st = 16; st >= 1; st >>= 1)
        if (__shfl_sync(0xffffffffu, excl, l + st) <= t) l += st;
      const int ax = __shfl_sync(0xffffffffu, xa, l) + t - __shfl_sync(0xffffffffu, excl, l);
      const int ay = __shfl_sync(0xffffffffu, by, l), az = __shfl_sync(0xffffffffu, bz, l);
      const int hx = h0 + ax, hy = h1 + ay, hz = h2 + az;
      const int li = (az * wy + ay) * wx + ax;
      int c = 0;
      if (t < total) {
        float dxf, dyf, dzf;
        c = classify_node(hx, hy, hz, im, dxf, dyf, dzf);
        if (c < 0) c = corner_count(g.dim, dxf, dyf, dzf, im.rSqf);
        if (c > 0) code[li] = (unsigned short)c;
      }
      const unsigned sm = __ballot_sync(0xffffffffu, c < 0);
      if (sm) {
        if (qn + 32 > SFC_QW) flush();
        if (c < 0) q[warp][qn + __popc(sm & ((1u << lane) - 1u))] = make_int4((int)blockIdx.x, li,
                                                                          hx | (hy << 16), hz);
        qn += __popc(sm);
        __syncwarp();
      }
    }
  }
  if (qn) flush();
}

// Exact double of a small non-negative integer without the conversion unit.
static __device__ __forceinline__ double small_int_to_double(int k) {
  return __hiloint2double(0x43300000, k) - 4503599627370496.0;  // 2^52 + k - 2^52
}

// One row of sub-cells whose FP32 decision is not certain: the row fixes
// sub-cell index ia on axis pa and ib on axis pb and runs over the 10
// indices c of the remaining axis.  Sub-cells whose FP32 c-term lies below
// the band count as inside, above it as outside, and the ones inside the
// band are decided with the reference's FP64 expressions
// (src/LBM_PSM_exchangeParticleData.cpp:144-168).  Kept out of line so that
// the rare branch calling it is not predicated into every row.
static __device__ __noinline__ int exact_row_count(const Img& im, int hx, int hy, int hz, int pa,
                                                   int pb, int ia, int ib, float dc, float tlo,
                                                   float thi) {
  const double sliceWidth = 1.0 / ((double)10);
  const double rSq = im.r * im.r;
  const double D[3] = {small_int_to_double(hx) - im.xl[0], small_int_to_double(hy) - im.xl[1],
                       small_int_to_double(hz) - im.xl[2]};
  int n = 0;
#pragma unroll
  for (int c = 0; c < 10; ++c) {
    const float t = dc + (float)(-0.5 + ((double)c + 0.5) * 0.1);
    const float sc = t * t;
    if (sc < tlo) {
      ++n;
    } else if (sc <= thi) {
      const int i0 = pa == 0 ? ia : (pb == 0 ? ib : c);
      const int i1 = pa == 1 ? ia : (pb == 1 ? ib : c);
      const int i2 = pa == 2 ? ia : (pb == 2 ? ib : c);
      const double t0 = D[0] + (-0.5 + (small_int_to_double(i0) + 0.5) * sliceWidth);
      const double t1 = D[1] + (-0.5 + (small_int_to_double(i1) + 0.5) * sliceWidth);
      const double t2 = D[2] + (-0.5 + (small_int_to_double(i2) + 0.5) * sliceWidth);
      const double ax = t0 * t0, ay = t1 * t1, az = t2 * t2;
      if (ax + ay + az < rSq) ++n;
    }
  }
  return n;
}

// The same for a whole 2-D node (10 x 10 sub-cells).
static __device__ __noinline__ int exact_count_2d(const Img& im, int hx, int hy) {
  const double sliceWidth = 1.0 / ((double)10);
  const double rSq = im.r * im.r;
  const double D0 = (double)hx - im.xl[0], D1 = (double)hy - im.xl[1];
  int n = 0;
  for (int a = 0; a < 10; ++a) {
    const double ta = D0 + (-0.5 + ((double)a + 0.5) * sliceWidth);
    const double ax = ta * ta;
    for (int b = 0; b < 10; ++b) {
      const double tb = D1 + (-0.5 + ((double)b + 0.5) * sliceWidth);
      if (ax + tb * tb < rSq) ++n;
    }
  }
  return n;
}

// Phase 2: sub-cell counts of the shell nodes, one node per lane, the list
// walked by a persistent grid in warp-sized chunks.
//
// 3-D: with the axes ordered so that the inner axis c has the smallest
// |offset| (its rows run most nearly along the sphere surface, so fewest of
// them cross it), a node's sub-cells are 10 slabs a of 100 rows (a, b).  A
// row whose 10 sub-cell sums are all below r^2 - M counts 10, one whose sums
// are all above r^2 + M counts 0 (M bounds the FP32 error, 16x the worst
// case); a row in between crosses the surface.  Each lane first tests its
// node's slabs as wholes: a slab whose largest row sum (its a-term plus the
// largest b-term) passes the inside test counts 100, one whose smallest
// fails the outside test counts 0 -- exactly what its rows would give, the
// FP32 sums being monotone in each term.  The other slabs go to a per-warp
// queue, taken one slab per lane: the slab's rows are tested and its
// crossing rows pushed into a per-warp buffer that is drained 32 rows at a
// time, one row per lane: the count is the rank of r^2 - M - s_ab among the
// node's 10 sorted c-terms, and a c-term within the margin band makes the
// row ambiguous, in which case that row alone is recounted exactly in FP64.
// 2-D: 100 sub-cells per node, counted in FP32 with the same margin; a node
// with any ambiguous sub-cell is recounted exactly.
__global__ void __launch_bounds__(SFS_THREADS, 8) sf_shell_kernel(MapParams p) {
  constexpr int NW = SFS_THREADS / 32;
  __shared__ float s_sorted[NW][32][17];  // 10 sorted c-terms + padding (odd stride)
  __shared__ float s_lo[NW][32];
  __shared__ float s_hi[NW][32];
  __shared__ int s_cnt[NW][32];
  __shared__ int s_ent[NW][32];   // shell-list entry of each lane's node
  __shared__ int s_perm[NW][32];  // its axis order: pa | pb << 2
  __shared__ float s_dc[NW][32];  // its inner-axis offset
  __shared__ float buf_s[NW][SFS_BUF];
  __shared__ unsigned short buf_o[NW][SFS_BUF];   // owner lane | a << 5 | b << 9
  __shared__ unsigned short q_slab[NW][32 * 10];  // partial slabs: owner lane | a << 5
  __shared__ float s_da[NW][32], s_db[NW][32], s_lin[NW][32], s_hout[NW][32];
  const unsigned long long tot = p.pair_total[2];
  const int total = (int)min(tot, (unsigned long long)p.shell_cap);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gw = blockIdx.x * NW + warp, nw = gridDim.x * NW;
  const float u = 5.9604644775390625e-08f;  // 2^-24
  const Geom& g = p.g;
#pragma unroll
  for (int k = 10; k < 16; ++k) s_sorted[warp][lane][k] = 3.0e38f;
  for (int base = gw * 32; base < total; base += nw * 32) {
    const int e = base + lane;
    const bool valid = e < total;
    const int4 ent = p.shell[valid ? e : base];
    const Img& im = p.img[ent.x];
    const int hx = ent.z & 0xFFFF, hy = ent.z >> 16, hz = ent.w;
    const float dxf = small_int_to_float(hx - im.xi[0]) - im.xf[0];
    const float dyf = small_int_to_float(hy - im.xi[1]) - im.xf[1];
    const float dzf = small_int_to_float(hz - im.xi[2]) - im.xf[2];
    const float rSqf = im.rSqf;
    int n = 0;
    if (g.dim == 2) {
      const float Ea = fabsf(dxf) + 2.0f, Eb = fabsf(dyf) + 2.0f;
      const float M = 16.0f * u * (Ea * Ea + Eb * Eb + rSqf);
      const float lo = rSqf - M, hi = rSqf + M;
      int amb = 0;
      for (int a = 0; a < 10; ++a) {
        const float ta = dxf + sub_offset(a);
        const float sa = ta * ta;
#pragma unroll
        for (int b = 0; b < 10; ++b) {
          const float tb = dyf + (float)(-0.5 + ((double)b + 0.5) * 0.1);
          const float t = sa + tb * tb;
          n += (t < lo);
          amb += (t >= lo) & (t <= hi);
        }
      }
      if (valid && amb) n = exact_count_2d(im, hx, hy);
    } else {
      // axis order: inner c along the smallest |offset| (its rows run most
      // nearly along the surface, so fewest cross it), outer a along the
      // largest (the surface crosses the node nearly perpendicular to it, so
      // fewest slabs are partial), middle b the other
      float da = dxf, db = dyf, dc = dzf;
      int pa = 0, pb = 1;
      {
        const float ax = fabsf(dxf), ay = fabsf(dyf), az = fabsf(dzf);
        if (ax <= ay && ax <= az) {
          da = dyf; db = dzf; dc = dxf; pa = 1; pb = 2;
        } else if (ay <= ax && ay <= az) {
          da = dxf; db = dzf; dc = dyf; pa = 0; pb = 2;
        }
        if (fabsf(db) > fabsf(da)) {  // outer and middle swap: sums and margins are symmetric
          const float t = da; da = db; db = t;
          const int q = pa; pa = pb; pb = q;
        }
      }
      const float Ea = fabsf(da) + 2.0f, Eb = fabsf(db) + 2.0f, Ec = fabsf(dc) + 2.0f;
      const float M = 16.0f * u * (Ea * Ea + Eb * Eb + Ec * Ec + rSqf);
      const float lo = rSqf - M, hi = rSqf + M;
      // the 10 c-terms, sorted (odd-even transposition)
      float sc[10];
#pragma unroll
      for (int c = 0; c < 10; ++c) {
        const float t = dc + (float)(-0.5 + ((double)c + 0.5) * 0.1);
        sc[c] = t * t;
      }
#pragma unroll
      for (int r = 0; r < 10; ++r) {
#pragma unroll
        for (int c = r & 1; c + 1 < 10; c += 2) {
          const float x = fminf(sc[c], sc[c + 1]), y = fmaxf(sc[c], sc[c + 1]);
          sc[c] = x;
          sc[c + 1] = y;
        }
      }
#pragma unroll
      for (int c = 0; c < 10; ++c) s_sorted[warp][lane][c] = sc[c];
      s_lo[warp][lane] = lo;
      s_hi[warp][lane] = hi;
      s_cnt[warp][lane] = 0;
      const float lo_in = lo - sc[9];   // row wholly inside: s_ab + max c-term < lo
      const float hi_out = hi - sc[0];  // row wholly outside: s_ab + min c-term > hi
      float sb_min = 3.0e38f, sb_max = 0.0f;
#pragma unroll
      for (int b = 0; b < 10; ++b) {
        const float t = db + sub_offset(b);
        const float v = t * t;
        sb_min = fminf(sb_min, v);
        sb_max = fmaxf(sb_max, v);
      }
      s_ent[warp][lane] = valid ? e : base;
      s_perm[warp][lane] = pa | (pb << 2);
      s_dc[warp][lane] = dc;
      s_da[warp][lane] = da;
      s_db[warp][lane] = db;
      s_lin[warp][lane] = lo_in;
      s_hout[warp][lane] = hi_out;
      // whole slabs: inside (100), outside (0), or partial (queued)
      unsigned pm = 0;
#pragma unroll
      for (int a = 0; a < 10; ++a) {
        const float ta = da + sub_offset(a);
        const float sa = ta * ta;
        const bool in = sa + sb_max < lo_in;
        const bool out = sa + sb_min > hi_out;
        n += in ? 100 : 0;
        pm |= (!in && !out) ? (1u << a) : 0u;
      }
      if (!valid) pm = 0;
      int nslab;
      {
        const int cnt = __popc(pm);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        int pos = incl - cnt;
        while (pm) {
          const int a = __ffs(pm) - 1;
          pm &= pm - 1u;
          q_slab[warp][pos++] = (unsigned short)(lane | (a << 5));
        }
        nslab = __shfl_sync(0xffffffffu, incl, 31);
      }
      __syncwarp();
      // count of one buffered crossing row, added to its owner lane
      auto drain_row = [&](int k) {
        const float sv = buf_s[warp][k];
        const int o = buf_o[warp][k];
        const int ow = o & 31;
        const float tlo = s_lo[warp][ow] - sv, thi = s_hi[warp][ow] - sv;
        const float* srt = s_sorted[warp][ow];
        int r = 0;  // number of c-terms below tlo (entries 10..15 are +huge)
        if (srt[r + 7] < tlo) r += 8;
        if (srt[r + 3] < tlo) r += 4;
        if (srt[r + 1] < tlo) r += 2;
        if (srt[r] < tlo) r += 1;
        int rc = r;
        if (srt[r] <= thi) {  // a c-term inside the margin band: decide it exactly
          const int4 oe = p.shell[s_ent[warp][ow]];
          const int pp = s_perm[warp][ow];
          rc = exact_row_count(p.img[oe.x], oe.z & 0xFFFF, oe.z >> 16, oe.w, pp & 3, pp >> 2,
                               (o >> 5) & 15, (o >> 9) & 15, s_dc[warp][ow], tlo, thi);
        }
        if (rc) atomicAdd(&s_cnt[warp][ow], rc);
      };
      int wtotal = 0;  // rows in the warp buffer (warp-uniform)
      for (int k0 = 0; k0 < nslab; k0 += 32) {
        // one partial slab per lane: its rows, the crossing ones buffered
        unsigned cm = 0;
        int ow = 0, a = 0;
        float sa = 0.0f;
        if (k0 + lane < nslab) {
          const int q = q_slab[warp][k0 + lane];
          ow = q & 31;
          a = q >> 5;
          const float ta = s_da[warp][ow] + sub_offset(a);
          sa = ta * ta;
          const float dbo = s_db[warp][ow], lin = s_lin[warp][ow], hout = s_hout[warp][ow];
          int in_rows = 0;
#pragma unroll
          for (int b = 0; b < 10; ++b) {
            const float tb = dbo + sub_offset(b);
            const float sv = sa + tb * tb;
            const bool inside = sv < lin;
            in_rows += inside ? 10 : 0;
            cm |= (!inside && sv <= hout) ? (1u << b) : 0u;
          }
          if (in_rows) atomicAdd(&s_cnt[warp][ow], in_rows);
        }
        // append the crossing rows to the warp buffer
        const int cnt = __popc(cm);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        int pos = wtotal + incl - cnt;
        if (cm) {
          const float dbo = s_db[warp][ow];
          while (cm) {
            const int b = __ffs(cm) - 1;
            cm &= cm - 1u;
            const float tb = dbo + sub_offset(b);
            buf_s[warp][pos] = sa + tb * tb;
            buf_o[warp][pos] = (unsigned short)(ow | (a << 5) | (b << 9));
            ++pos;
          }
        }
        wtotal += __shfl_sync(0xffffffffu, incl, 31);
        __syncwarp();
        // drain 32 rows at a time, one per lane
        while (wtotal >= 32) {
          drain_row(wtotal - 32 + lane);
          wtotal -= 32;
          __syncwarp();
        }
      }
      if (lane < wtotal) drain_row(lane);
      __syncwarp();
      n += s_cnt[warp][lane];
      __syncwarp();
    }
    if (valid) p.sfcode[im.sf_off + ent.y] = (unsigned short)n;
  }
}

// Phase 2 of the map, per node: the images whose boxes contain it, in image
// order (the cell list is sorted), through the update of setParticlesOnLattice
// (src/LBM_PSM_exchangeParticleData.cpp:69-106) on the two-slot table
// (setParticleOnLattice / setToZero, src/LBM_PSM_lattice.cpp:257-324).
// decFlag = (sf > 1e-5) + 2*(sf_old > 1e-5): cases 0 and 2 clear the tag's slot
// (case 0 finds none unless the tag is the empty marker 0), cases 1 and 3 set
// it (case 3's condition sf > sf_old || id_old == tag holds because
// sf_old > 1e-5 means the tag matched), so only the sf bit decides.  sf > 1e-5
// exactly when the code is non-zero.  The table is written back only where it
// changed.
// Bit equality of two doubles as two 32-bit compares (64-bit integer
// compares take the slow path on this GPU).
static __device__ __forceinline__ bool same_bits(double a, double b) {
  return __double2loint(a) == __double2loint(b) && __double2hiint(a) == __double2hiint(b);
}

// FP64 storage: the table in FP64 (ids, eps, us) with the FP32 mirror.
__global__ void __launch_bounds__(512) node_apply_kernel(MapParams p) {
  const int c = (blockIdx.z * p.C[1] + blockIdx.y) * p.C[0] + blockIdx.x;
  const int cnt = p.cell_count[c];
  if (cnt == 0) return;
  if (p.pair_total[0] > (unsigned long long)p.list_cap ||
      p.pair_total[1] > (unsigned long long)p.sf_cap)
    return;
  const Geom& g = p.g;
  const int sx = blockIdx.x * p.cb[0] + threadIdx.x;
  const int sy = blockIdx.y * p.cb[1] + threadIdx.y;
  const int sz = blockIdx.z * p.cb[2] + threadIdx.z;
  if (sx >= g.S[0] || sy >= g.S[1] || sz >= g.S[2]) return;
  const long long n = node_index(g, sx, sy, sz);
  const int hi = sx + g.off[0], hj = sy + g.off[1];
  const int hk = sz - box_of_z(g, sz) * g.bz + g.off[2];  // z in the box's own frame
  const int* lst = p.list + p.cell_off[c];
  int id[2] = {0, 0};
  double eps[2] = {0.0, 0.0};
  bool have_ids = false, have_eps = false, ids_dirty = false;
  bool slot_dirty[2] = {false, false};
  double us[6];
  for (int t = 0; t < cnt; ++t) {
    const Img& im = p.img[lst[t]];
    if (sx < im.lo[0] || sx >= im.hi[0] || sy < im.lo[1] || sy >= im.hi[1] || sz < im.lo[2] ||
        sz >= im.hi[2])
      continue;
    const int li = ((sz - im.lo[2]) * im.box[1] + (sy - im.lo[1])) * im.box[0] + (sx - im.lo[0]);
    const unsigned short cd = p.sfcode[im.sf_off + li];
    const int tag = im.tag;
    if (!have_ids) {
      const int2 v = p.tab.ids[n];
      id[0] = v.x;
      id[1] = v.y;
      have_ids = true;
    }
    const int match = tag == id[0] ? 0 : (tag == id[1] ? 1 : -1);
    if (cd == 0) {  // setToZero (src/LBM_PSM_lattice.cpp:302-324)
      if (match >= 0) {
        if (!have_eps) {
          const double2 e = p.tab.eps[n];
          eps[0] = e.x;
          eps[1] = e.y;
          have_eps = true;
        }
        id[match] = 0;
        eps[match] = 0.0;
        us[3 * match] = us[3 * match + 1] = us[3 * match + 2] = 0.0;
        ids_dirty = true;
        slot_dirty[match] = true;
      }
      continue;
    }
    // setParticleOnLattice: matching slot, else the first empty one, else drop
    int slot = -1;
    if (id[0] == tag)
      slot = 0;
    else if (id[1] == tag)
      slot = 1;
    else if (id[0] == 0)
      slot = 0;
    else if (id[1] == 0)
      slot = 1;
    if (slot < 0) continue;
    if (!have_eps) {
      const double2 e = p.tab.eps[n];
      eps[0] = e.x;
      eps[1] = e.y;
      have_eps = true;
    }
    const double sf = cd == SF_ONE ? 1.0 : p.sf_value[cd];
    // rigid-body velocity of the node (src/LBM_PSM_exchangeParticleData.cpp:83-89)
    double u0, u1, u2;
    if (im.has_spin) {
      const double dx = (double)hi - im.xl[0];
      const double dy = (double)hj - im.xl[1];
      const double dz = (double)hk - im.xl[2];
      u0 = im.uT[0] + im.om[1] * dz - im.om[2] * dy;
      u1 = im.uT[1] + im.om[2] * dx - im.om[0] * dz;
      u2 = im.uT[2] + im.om[0] * dy - im.om[1] * dx;
    } else {
      // every omega component +0.0 and no uT component -0.0: the reference's
      // (uT + 0*dz) - 0*dy is uT bit for bit
      u0 = im.uT[0];
      u1 = im.uT[1];
      u2 = im.uT[2];
    }
    // re-setting a slot to the values it already holds changes nothing
    bool same = !slot_dirty[slot] && id[slot] == tag && same_bits(eps[slot], sf);
    if (same) {
      const double* cur = p.tab.us + 6 * n + 3 * slot;
      same = same_bits(cur[0], u0) && same_bits(cur[1], u1) && same_bits(cur[2], u2);
    }
    if (!same) {
      if (id[slot] != tag) ids_dirty = true;
      id[slot] = tag;
      eps[slot] = sf;
      us[3 * slot + 0] = u0;
      us[3 * slot + 1] = u1;
      us[3 * slot + 2] = u2;
      slot_dirty[slot] = true;
    }
  }
  if (ids_dirty) {
    p.tab.ids[n] = make_int2(id[0], id[1]);
    p.tab.flag[n] = (uint8_t)((id[0] > 0 ? 1 : 0) | (id[1] > 0 ? 2 : 0));
  }
  if (slot_dirty[0] || slot_dirty[1]) p.tab.eps[n] = make_double2(eps[0], eps[1]);
  for (int b = 0; b < 2; ++b) {
    if (!slot_dirty[b]) continue;
    for (int k = 0; k < 3; ++k) p.tab.us[6 * n + 3 * b + k] = us[3 * b + k];
    if (p.write32)
      p.tab.rec32[2 * n + b] = make_float4((float)eps[b], (float)us[3 * b], (float)us[3 * b + 1],
                                           (float)us[3 * b + 2]);
  }
}


// FP32 / FP16 storage: the table is ids + the FP32 records the collide
// kernel reads (eps, u_s per slot); the same update rules, no FP64.  The
// records hold the FP32 roundings of the reference's values (for spinning
// images the node velocity is formed in FP32).
//
// One node's update state: the tags of its two slots as they stand after
// the images applied so far.  Slot records are written through (the table
// ends with the same records as when only changed ones are written, without
// a read before the write), so only the ids live in registers; the ids and
// the flag are written back at the end if they changed.
struct Apply32 {
  int id0, id1;
  bool ids_dirty;

  __device__ __forceinline__ void init(int2 ids) {
    id0 = ids.x;
    id1 = ids.y;
    ids_dirty = false;
  }

  // one image with code cd at node n; nv.yzw is the node velocity it sets
  __device__ __forceinline__ void image(const MapParams& p, long long n, int tag,
                                        unsigned short cd, float4 nv) {
    if (cd == 0) {  // setToZero (src/LBM_PSM_lattice.cpp:302-324)
      const int m = tag == id0 ? 0 : (tag == id1 ? 1 : -1);
      if (m >= 0) {
        if (m == 0) id0 = 0; else id1 = 0;
        ids_dirty = true;
        p.tab.rec32[2 * n + m] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      return;
    }
    // setParticleOnLattice: matching slot, else the first empty one, else drop
    int slot = -1;
    if (id0 == tag)
      slot = 0;
    else if (id1 == tag)
      slot = 1;
    else if (id0 == 0)
      slot = 0;
    else if (id1 == 0)
      slot = 1;
    if (slot < 0) return;
    nv.x = cd == SF_ONE ? 1.0f : p.sf_value32[cd];
    const int cur = slot == 0 ? id0 : id1;
    if (cur != tag) {
      if (slot == 0) id0 = tag; else id1 = tag;
      ids_dirty = true;
    }
    // written whether or not it changes: a store does not wait, whereas
    // reading the record first to skip an unchanged one would
    p.tab.rec32[2 * n + slot] = nv;
  }

  __device__ __forceinline__ void store(const MapParams& p, long long n) const {
    if (ids_dirty) {
      p.tab.ids[n] = make_int2(id0, id1);
      p.tab.flag[n] = (uint8_t)((id0 > 0 ? 1 : 0) | (id1 > 0 ? 2 : 0));
    }
  }
};

// rigid-body velocity of node (hi, hj, hk) of a spinning image, in FP32
// (src/LBM_PSM_exchangeParticleData.cpp:83-89)
static __device__ __forceinline__ float4 spin_velocity(const Img& im, int hi, int hj, int hk) {
  const float dx = small_int_to_float(hi - im.xi[0]) - im.xf[0];
  const float dy = small_int_to_float(hj - im.xi[1]) - im.xf[1];
  const float dz = small_int_to_float(hk - im.xi[2]) - im.xf[2];
  return make_float4(0.f, im.uTf[0] + im.omf[1] * dz - im.omf[2] * dy,
                     im.uTf[1] + im.omf[2] * dx - im.omf[0] * dz,
                     im.uTf[2] + im.omf[0] * dy - im.omf[1] * dx);
}

// NPT nodes per thread (z, z + blockDim.z, ... within the cell; one node in
// 2-D) of a cell that some image box touches.  The images of the cell's list
// are visited in image order through their compact records, which cell_sort
// copied next to the list entries (three 16-byte loads straight after the
// cell's offset, instead of list index, then record, then the scattered
// fields of Img), each record serving all the thread's nodes, whose code
// and slot record loads are independent.  The slot ids are loaded with the
// cell's count and offset, so that they add no round of dependent loads.
template <int NPT>
__global__ void __launch_bounds__(512 / NPT, 8) node_apply32_kernel(MapParams p) {
  const int c = (blockIdx.z * p.C[1] + blockIdx.y) * p.C[0] + blockIdx.x;
  const Geom& g = p.g;
  const int sx = blockIdx.x * p.cb[0] + threadIdx.x;
  const int sy = blockIdx.y * p.cb[1] + threadIdx.y;
  const int sz0 = blockIdx.z * p.cb[2] + threadIdx.z;
  const int dz = (int)blockDim.z;
  const long long n0 = node_index(g, sx, sy, sz0);
  const long long zstride = (long long)dz * g.P0 * g.S[1];
  const bool inside = sx < g.S[0] && sy < g.S[1] && sz0 < g.S[2];
  bool has[NPT];
#pragma unroll
  for (int k = 0; k < NPT; ++k)
    has[k] = inside && (int)threadIdx.z + k * dz < p.cb[2] && sz0 + k * dz < g.S[2];
  // the cell's count and offset, the overflow words and the slot ids of the
  // thread's nodes: independent loads, issued together
  const int cnt = __ldg(p.cell_count + c);
  const int coff = __ldg(p.cell_off + c);
  const unsigned long long tot0 = __ldg(p.pair_total), tot1 = __ldg(p.pair_total + 1);
  int2 ids0[NPT];
#pragma unroll
  for (int k = 0; k < NPT; ++k)
    ids0[k] = has[k] && cnt ? p.tab.ids[n0 + k * zstride] : make_int2(0, 0);
  if (cnt == 0 || !inside) return;
  if (tot0 > (unsigned long long)p.list_cap || tot1 > (unsigned long long)p.sf_cap) return;
  const int4* __restrict__ lrec = p.lrec + 3 * (long long)coff;
  Apply32 st[NPT];
#pragma unroll
  for (int k = 0; k < NPT; ++k) st[k].init(ids0[k]);
  bool touched[NPT];
#pragma unroll
  for (int k = 0; k < NPT; ++k) touched[k] = false;
  for (int t = 0; t < cnt; ++t) {
    const int4 A = __ldg(lrec + 3 * t);
    const unsigned ax = (unsigned)A.x, ay = (unsigned)A.y, az = (unsigned)A.z;
    const int lo0 = (int)(ax & 0xFFFFu), lo1 = (int)(ay & 0xFFFFu), lo2 = (int)(az & 0xFFFFu);
    const int hi2 = (int)(az >> 16);
    if (sx < lo0 || sx >= (int)(ax >> 16) || sy < lo1 || sy >= (int)(ay >> 16)) continue;
    bool in[NPT];
    bool any = false;
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
      const int z = sz0 + k * dz;
      in[k] = has[k] && z >= lo2 && z < hi2;
      any = any || in[k];
    }
    if (!any) continue;
    const int4 B = __ldg(lrec + 3 * t + 1);
    const int4 U = __ldg(lrec + 3 * t + 2);
    const unsigned bz = (unsigned)B.z;
    const int bx = (int)(bz & 0xFFFFu), by = (int)(bz >> 16);
    const long long off = (long long)(((unsigned long long)(unsigned)B.y << 32) |
                                      (unsigned long long)(unsigned)B.x) +
                          (long long)(sy - lo1) * bx + (sx - lo0);
    const long long plane = (long long)by * bx;
    unsigned short cd[NPT];
#pragma unroll
    for (int k = 0; k < NPT; ++k)
      cd[k] = in[k] ? __ldg(p.sfcode + off + (sz0 + k * dz - lo2) * plane) : (unsigned short)0;
#pragma unroll
    for (int k = 0; k < NPT; ++k) touched[k] = touched[k] || in[k];
    if (B.w) {
      const int hi = sx + g.off[0], hj = sy + g.off[1];
#pragma unroll
      for (int k = 0; k < NPT; ++k) {
        if (!in[k]) continue;
        const int z = sz0 + k * dz;
        const int hk = z - box_of_z(g, z) * g.bz + g.off[2];  // z in the box's own frame
        st[k].image(p, n0 + k * zstride, A.w, cd[k], spin_velocity(p.img[U.w], hi, hj, hk));
      }
    } else {
      const float4 nv = make_float4(0.f, __int_as_float(U.x), __int_as_float(U.y),
                                    __int_as_float(U.z));
#pragma unroll
      for (int k = 0; k < NPT; ++k)
        if (in[k]) st[k].image(p, n0 + k * zstride, A.w, cd[k], nv);
    }
  }
#pragma unroll
  for (int k = 0; k < NPT; ++k)
    if (touched[k]) st[k].store(p, n0 + k * zstride);
}

// img_prep; then two independent chains: the cell lists (scan, fill, sort)
// and the solid fractions (classify, shell); then the table update, which
// needs both.  With an aux stream the cell-list chain runs there.
cudaError_t launch_map(const MapParams& p, cudaStream_t st, cudaStream_t aux, cudaEvent_t fork,
                       cudaEvent_t join) {
  if (p.n <= 0) return cudaSuccess;
  const int ncells = p.C[0] * p.C[1] * p.C[2];
  const int tb = 128;
  const unsigned wblocks = (unsigned)(((long long)p.n * 32 + tb - 1) / tb);
  // IMG_LANES images per block, spread over as many multiprocessors as possible
  img_prep_kernel<<<(p.n + IMG_LANES - 1) / IMG_LANES, IMG_LANES, 0, st>>>(p);
  const bool two = aux && fork && join;
  cudaStream_t cl = two ? aux : st;
  cudaError_t e;
  if (two) {
    if ((e = cudaEventRecord(fork, st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(aux, fork, 0)) != cudaSuccess) return e;
  }
  cell_scan_kernel<<<1, SCAN_THREADS, 0, cl>>>(p.cell_count, p.cell_off, ncells);
  img_fill_kernel<<<wblocks, tb, 0, cl>>>(p);
  cell_sort_kernel<<<(ncells + 255) / 256, 256, 0, cl>>>(p, ncells);
  sf_classify_kernel<<<p.n, SFC_THREADS, 0, st>>>(p);
  sf_shell_kernel<<<p.sm_count * 8, SFS_THREADS, 0, st>>>(p);
  if (two) {
    if ((e = cudaEventRecord(join, aux)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(st, join, 0)) != cudaSuccess) return e;
  }
  dim3 block(p.cb[0], p.cb[1], p.cb[2]);
  dim3 cells((unsigned)p.C[0], (unsigned)p.C[1], (unsigned)p.C[2]);
  if (p.write32) {
    constexpr int NPT = 2;  // nodes per thread along z
    dim3 part(p.cb[0], p.cb[1], (p.cb[2] + NPT - 1) / NPT);
    node_apply32_kernel<NPT><<<cells, part, 0, st>>>(p);
  } else {
    node_apply_kernel<<<cells, block, 0, st>>>(p);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------------ reduce
constexpr int RED_THREADS = 128;

// Node (i, j, k) lies beyond the early-out radius rP of the image for
// certain (FP32 distance with the margin proven for classify_node), so its
// solid fraction for this image is 0.
static __device__ __forceinline__ bool beyond_rP(const Img& im, int i, int j, int k) {
  const float u = 5.9604644775390625e-08f;  // 2^-24
  const float dx = small_int_to_float(i - im.xi[0]) - im.xf[0];
  const float dy = small_int_to_float(j - im.xi[1]) - im.xf[1];
  const float dz = small_int_to_float(k - im.xi[2]) - im.xf[2];
  const float d32 = dx * dx + dy * dy + dz * dz;
  const float m = 16.0f * u * (5.0f * d32 + 2.0f * (fabsf(dx) + fabsf(dy) + fabsf(dz)) + 1.0f + im.rP2f);
  return d32 > im.rP2f + m;
}

// The step's status word into host memory for the host-pointer step (every
// kernel that sets a bit ran before the reduction in stream order).
static __device__ __forceinline__ void copy_status(const ReduceParams& p) {
  if (p.status_out && blockIdx.x == 0 && threadIdx.x == 0)
    *p.status_out = *static_cast<const volatile int*>(p.status);
}

static __device__ __forceinline__ void block_reduce_store(double (&acc)[12], const ReduceParams& p,
                                                          int ip) {
  // fixed-order reduction: butterfly within warps, then warps in index order
#pragma unroll
  for (int k = 0; k < 12; ++k)
    for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
  __shared__ double part[RED_THREADS / 32][12];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int k = 0; k < 12; ++k) part[warp][k] = acc[k];
  __syncthreads();
  if (threadIdx.x < 12) {
    const int k = threadIdx.x;
    double sum = 0.0;
    for (int w = 0; w < RED_THREADS / 32; ++w) sum += part[w][k];
    if (k < 3) {
      p.fh[3 * ip + k] = sum;
      if (p.fh2) p.fh2[3 * ip + k] = sum;
    } else if (k < 6) {
      p.th[3 * ip + (k - 3)] = sum;
      if (p.th2) p.th2[3 * ip + (k - 3)] = sum;
    } else {
      p.S[6 * ip + (k - 6)] = -sum;
      if (p.S2) p.S2[6 * ip + (k - 6)] = -sum;
    }
  }
}

// FP64 node forces (FP64 storage): the reference's per-node terms in FP64.
__global__ void __launch_bounds__(RED_THREADS) reduce_f64_kernel(ReduceParams p) {
  const int ip = blockIdx.x;
  const Geom& g = p.g;
  const int tag = p.tag[ip];
  const Img& bx = p.img[ip];  // box and centre from the map's image record
  const int wx = bx.qhi[0] - bx.qlo[0], wy = bx.qhi[1] - bx.qlo[1], wz = bx.qhi[2] - bx.qlo[2];
  double acc[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) acc[k] = 0.0;
  if (wx > 0 && wy > 0 && wz > 0) {
    const long long total = (long long)wx * wy * wz;
    const double ff = p.box[bx.bidx].forceFactor, tf = p.box[bx.bidx].torqueFactor;
    const double* nodeF = static_cast<const double*>(p.tab.nodeF);
    // x fastest: consecutive threads read consecutive nodes
    const FastDiv fx = make_fastdiv((unsigned)wx), fy = make_fastdiv((unsigned)wy);
    for (long long t = threadIdx.x; t < total; t += RED_THREADS) {
      const int q1 = (int)fast_div((unsigned)t, fx);
      const int q2 = (int)fast_div((unsigned)q1, fy);
      const int i = bx.qlo[0] + (int)t - q1 * wx;
      const int j = bx.qlo[1] + q1 - q2 * wy;
      const int k = bx.qlo[2] + q2;
      if (bx.solo && beyond_rP(bx, i, j, k)) continue;
      const long long n = node_index(g, i - g.off[0], j - g.off[1], k - g.off[2] + bx.zoff);
      const int2 id = p.tab.ids[n];
      int slot;
      if (tag == id.x)
        slot = 0;
      else if (tag == id.y)
        slot = 1;
      else
        continue;
      const double* nf = nodeF + 6 * n + 3 * slot;
      const double F0 = nf[0], F1 = nf[1], F2 = nf[2];
      acc[0] += F0 * ff;
      acc[1] += F1 * ff;
      acc[2] += F2 * ff;
      const double dx = (double)i - bx.xl[0];
      const double dy = (double)j - bx.xl[1];
      const double dz = (double)k - bx.xl[2];
      acc[3] += (dy * F2 - dz * F1) * tf;
      acc[4] += (dz * F0 - dx * F2) * tf;
      acc[5] += (dx * F1 - dy * F0) * tf;
      // 0.5*(a*b + a*b) is exactly a*b: doubling and halving are exact
      acc[6] += (dx * F0) * tf;
      acc[7] += (dy * F1) * tf;
      acc[8] += (dz * F2) * tf;
      acc[9] += 0.5 * (dy * F0 + dx * F1) * tf;
      acc[10] += 0.5 * (dz * F0 + dx * F2) * tf;
      acc[11] += 0.5 * (dz * F1 + dy * F2) * tf;
    }
  }
  block_reduce_store(acc, p, ip);
  copy_status(p);
}

// Error-free transformation: a + b = s + e exactly (Knuth's TwoSum; no
// contraction or reassociation under -fmad=false).
static __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// FP32 node forces (FP32 / FP16 / BF16 storage): per-node terms in FP32 (the
// node forces carry FP32 precision), accumulated per particle in double-float
// (hi + lo pairs combined with TwoSum, ~48-bit significand) on the FP32 pipe,
// then the per-warp results summed in FP64.  (FP64 arithmetic runs at 1/64 of
// the FP32 rate on this GPU.)  Issue- and latency-bound: 64 registers,
// 64-thread blocks (16 per multiprocessor: the 2281 images of the 256^3
// suspension run in one wave), two nodes'
// loads in flight per thread, and only the nodes of each row that may lie
// within rP visited (a sphere holds about half of its box), without the
// divergence of testing every box node.  The order of the sums is fixed by
// the image's box alone, so the results are reproducible bit for bit.
constexpr int RED_U = 2;
constexpr int RED32_THREADS = 64;  // FP32 reduction block
__global__ void __launch_bounds__(RED32_THREADS, 16) reduce_f32_kernel(ReduceParams p) {
  const int ip = blockIdx.x;
  const Geom& g = p.g;
  const int tag = p.tag[ip];
  const Img& bx = p.img[ip];  // box and centre from the map's image record
  const int wx = bx.qhi[0] - bx.qlo[0], wy = bx.qhi[1] - bx.qlo[1], wz = bx.qhi[2] - bx.qlo[2];
  float hi[12], lo[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) hi[k] = lo[k] = 0.0f;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (wx > 0 && wy > 0 && wz > 0) {
    const int xi[3] = {bx.xi[0], bx.xi[1], bx.xi[2]};  // xl = xi + xf exactly
    const float xf[3] = {bx.xf[0], bx.xf[1], bx.xf[2]};
    const float* nodeF = static_cast<const float*>(p.tab.nodeF);
    const int R = wy * wz;  // x-rows of the box
    const FastDiv fy = make_fastdiv((unsigned)wy);
    // A solo image's tag can only sit on nodes within rP (eps > 0 from this
    // image), so each row is cut to the x-range that may lie within rP: an
    // FP32 bound widened by 0.01 node, a superset (extra nodes fail the tag
    // test).  Each warp takes 32 rows at a time, one per lane, and walks the
    // nodes of their segments 32 at a time (x fastest, consecutive lanes on
    // consecutive nodes); a lane finds its node's row by a binary search of
    // the segments' offsets across the warp.
    const float rem0 = bx.rP2f * 1.0001f + 0.01f;
    for (int r0 = warp * 32; r0 < R; r0 += RED32_THREADS) {
      const int r = r0 + lane;
      int xa = bx.qlo[0], len = 0, j = 0, k = 0;
      if (r < R) {
        const int q = (int)fast_div((unsigned)r, fy);
        j = bx.qlo[1] + r - q * wy;
        k = bx.qlo[2] + q;
        int xb = bx.qhi[0];
        if (bx.solo) {
          const float dy = small_int_to_float(j - xi[1]) - xf[1];
          const float dz = small_int_to_float(k - xi[2]) - xf[2];
          const float rem = rem0 - dy * dy - dz * dz;
          if (rem < 0.0f) {
            xb = xa;
          } else {
            const float h = sqrtf(rem) + 0.01f;
            xa = max(xa, xi[0] + (int)ceilf(xf[0] - h));
            xb = min(xb, xi[0] + (int)floorf(xf[0] + h) + 1);
          }
        }
        len = max(xb - xa, 0);
      }
      int incl = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      const int excl = incl - len;
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      // RED_U nodes per lane and round, loaded before any is summed
      for (int base = 0; base < total; base += RED_U * 32) {
        int2 id[RED_U];
        float2 f01[RED_U], f23[RED_U], f45[RED_U];
        float dx[RED_U], dy[RED_U], dz[RED_U];
        bool ok[RED_U];
#pragma unroll
        for (int u = 0; u < RED_U; ++u) {
          const int t = base + u * 32 + lane;
          // the row holding node t: the last lane whose offset is <= t (a
          // row of length 0 shares its offset with the next row)
          int l = 0;
#pragma unroll
          for (int st = 16; st >= 1; st >>= 1)
            if (__shfl_sync(0xffffffffu, excl, l + st) <= t) l += st;
          const int ra = __shfl_sync(0xffffffffu, xa, l);
          const int re = __shfl_sync(0xffffffffu, excl, l);
          const int jj = __shfl_sync(0xffffffffu, j, l);
          const int kk = __shfl_sync(0xffffffffu, k, l);
          const int i = ra + t - re;
          ok[u] = t < total;
          id[u] = make_int2(0, 0);
          f01[u] = f23[u] = f45[u] = make_float2(0.f, 0.f);
          dx[u] = small_int_to_float(i - xi[0]) - xf[0];
          dy[u] = small_int_to_float(jj - xi[1]) - xf[1];
          dz[u] = small_int_to_float(kk - xi[2]) - xf[2];
          if (ok[u]) {
            const long long n = node_index(g, i - g.off[0], jj - g.off[1], kk - g.off[2] + bx.zoff);
            // both slots' forces are loaded with the ids (no second dependent load)
            id[u] = p.tab.ids[n];
            const float2* nf2 = reinterpret_cast<const float2*>(nodeF + 6 * n);
            f01[u] = nf2[0];
            f23[u] = nf2[1];
            f45[u] = nf2[2];
          }
        }
#pragma unroll
        for (int u = 0; u < RED_U; ++u) {
          if (!ok[u]) continue;
          float F0, F1, F2;
          if (tag == id[u].x) {
            F0 = f01[u].x;
            F1 = f01[u].y;
            F2 = f23[u].x;
          } else if (tag == id[u].y) {
            F0 = f23[u].y;
            F1 = f45[u].x;
            F2 = f45[u].y;
          } else {
            continue;
          }
          const float term[12] = {F0,
                                  F1,
                                  F2,
                                  dy[u] * F2 - dz[u] * F1,
                                  dz[u] * F0 - dx[u] * F2,
                                  dx[u] * F1 - dy[u] * F0,
                                  dx[u] * F0,
                                  dy[u] * F1,
                                  dz[u] * F2,
                                  0.5f * (dy[u] * F0 + dx[u] * F1),
                                  0.5f * (dz[u] * F0 + dx[u] * F2),
                                  0.5f * (dz[u] * F1 + dy[u] * F2)};
#pragma unroll
          for (int q = 0; q < 12; ++q) {
            float sv, e;
            two_sum(hi[q], term[q], sv, e);
            hi[q] = sv;
            lo[q] += e;
          }
        }
      }
    }
  }
  // fixed-order double-float reduction within the warp: the first two levels
  // halve the terms each lane carries (12 -> 6 -> 3, partners keeping
  // complementary halves), the last three are a butterfly on three terms
  const bool up16 = (lane & 16) != 0, up8 = (lane & 8) != 0;
  float h6[6], l6[6], h3[3], l3[3];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const float sh = up16 ? hi[k] : hi[k + 6], sl = up16 ? lo[k] : lo[k + 6];
    const float mh = up16 ? hi[k + 6] : hi[k], ml = up16 ? lo[k + 6] : lo[k];
    const float rh = __shfl_xor_sync(0xffffffffu, sh, 16);
    const float rl = __shfl_xor_sync(0xffffffffu, sl, 16);
    float sv, e;
    two_sum(mh, rh, sv, e);
    h6[k] = sv;
    l6[k] = ml + rl + e;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float sh = up8 ? h6[k] : h6[k + 3], sl = up8 ? l6[k] : l6[k + 3];
    const float mh = up8 ? h6[k + 3] : h6[k], ml = up8 ? l6[k + 3] : l6[k];
    const float rh = __shfl_xor_sync(0xffffffffu, sh, 8);
    const float rl = __shfl_xor_sync(0xffffffffu, sl, 8);
    float sv, e;
    two_sum(mh, rh, sv, e);
    h3[k] = sv;
    l3[k] = ml + rl + e;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
      const float h2 = __shfl_xor_sync(0xffffffffu, h3[k], o);
      const float l2 = __shfl_xor_sync(0xffffffffu, l3[k], o);
      float sv, e;
      two_sum(h3[k], h2, sv, e);
      h3[k] = sv;
      l3[k] = l3[k] + l2 + e;
    }
  }
  // warps in index order, still in double-float; one FP64 sum per term
  __shared__ float part_hi[RED32_THREADS / 32][12], part_lo[RED32_THREADS / 32][12];
  if ((lane & 7) == 0) {  // lanes 0, 8, 16, 24 hold terms 0-2, 3-5, 6-8, 9-11
    const int q0 = (up16 ? 6 : 0) + (up8 ? 3 : 0);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      part_hi[warp][q0 + k] = h3[k];
      part_lo[warp][q0 + k] = l3[k];
    }
  }
  __syncthreads();
  if (threadIdx.x < 12) {
    const int q = threadIdx.x;
    float sh = 0.0f, sl = 0.0f;
    for (int w = 0; w < RED32_THREADS / 32; ++w) {
      float sv, e;
      two_sum(sh, part_hi[w][q], sv, e);
      sh = sv;
      sl = sl + part_lo[w][q] + e;
    }
    const double sum = (double)sh + (double)sl;
    if (q < 3) {
      const double v = sum * p.box[bx.bidx].forceFactor;
      p.fh[3 * ip + q] = v;
      if (p.fh2) p.fh2[3 * ip + q] = v;
    } else if (q < 6) {
      const double v = sum * p.box[bx.bidx].torqueFactor;
      p.th[3 * ip + (q - 3)] = v;
      if (p.th2) p.th2[3 * ip + (q - 3)] = v;
    } else {
      const double v = -(sum * p.box[bx.bidx].torqueFactor);
      p.S[6 * ip + (q - 6)] = v;
      if (p.S2) p.S2[6 * ip + (q - 6)] = v;
    }
  }
  copy_status(p);
}

cudaError_t launch_reduce(const ReduceParams& p, cudaStream_t st) {
  if (p.n <= 0) return cudaSuccess;
  if (p.nodeF_is_double)
    reduce_f64_kernel<<<p.n, RED_THREADS, 0, st>>>(p);
  else
    reduce_f32_kernel<<<p.n, RED32_THREADS, 0, st>>>(p);
  return cudaGetLastError();
}

// the kernels whose parameters a replayed device-step graph updates per call
const void* img_prep_fn() { return (const void*)img_prep_kernel; }
const void* reduce_fn(int nodeF_is_double) {
  return nodeF_is_double ? (const void*)reduce_f64_kernel : (const void*)reduce_f32_kernel;
}

// ------------------------------------------------------------------ exports
// particle table in the reference layout (halo nodes of periodic axes empty)
__global__ void table_export_kernel(Geom g, Table t, int* ids, double* eps, double* us) {
  const long long total = (long long)g.L[0] * g.L[1] * g.L[2];
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= total) return;
  const int k = (int)(r % g.L[2]);
  const int j = (int)((r / g.L[2]) % g.L[1]);
  const int i = (int)(r / ((long long)g.L[2] * g.L[1]));
  const int sx = i - g.off[0], sy = j - g.off[1], sz = k - g.off[2];
  const bool ok = sx >= 0 && sx < g.S[0] && sy >= 0 && sy < g.S[1] && sz >= 0 && sz < g.S[2];
  int2 id = make_int2(0, 0);
  double2 e = make_double2(0.0, 0.0);
  double u[6] = {0, 0, 0, 0, 0, 0};
  if (ok) {
    const long long n = node_index(g, sx, sy, sz);
    id = t.ids[n];
    if (t.eps) {
      e = t.eps[n];
      for (int c = 0; c < 6; ++c) u[c] = t.us[6 * n + c];
    } else {  // FP32 / FP16 storage keeps only the FP32 records
      const float4 r0 = t.rec32[2 * n], r1 = t.rec32[2 * n + 1];
      e = make_double2(r0.x, r1.x);
      u[0] = r0.y; u[1] = r0.z; u[2] = r0.w;
      u[3] = r1.y; u[4] = r1.z; u[5] = r1.w;
    }
  }
  if (ids) {
    ids[2 * r] = id.x;
    ids[2 * r + 1] = id.y;
  }
  if (eps) {
    eps[2 * r] = e.x;
    eps[2 * r + 1] = e.y;
  }
  if (us)
    for (int c = 0; c < 6; ++c) us[6 * r + c] = u[c];
}

cudaError_t launch_table_export(const Geom& g, const Table& t, int* ids, double* eps, double* us,
                                cudaStream_t st) {
  const long long total = (long long)g.L[0] * g.L[1] * g.L[2];
  table_export_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(g, t, ids, eps, us);
  return cudaGetLastError();
}

// execute_write_vti field read (src/fix_LBM_PSM_writeVTI.h:146-169)
__global__ void export_fields_kernel(Geom g, Table t, const double* rho, const double* u,
                                     int as_double, double B0, double rho0, double u0,
                                     void* solid_out, void* rho_out, void* u_out) {
  const int nxi = g.L[0] - 2, nyi = g.L[1] - 2, nzi = g.dim == 3 ? g.L[2] - 2 : 1;
  const long long total = (long long)nxi * nyi * nzi;
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= total) return;
  const int i = 1 + (int)(id % nxi);
  const int j = 1 + (int)((id / nxi) % nyi);
  const int k = (g.dim == 3 ? 1 : 0) + (int)(id / ((long long)nxi * nyi));
  const int sx = i - g.off[0], sy = j - g.off[1], sz = k - g.off[2];
  const long long n = node_index(g, sx, sy, sz);
  const double2 e = t.eps ? t.eps[n] : make_double2(t.rec32[2 * n].x, t.rec32[2 * n + 1].x);
  const double Bv = (e.x + e.y);
  const double sv = (Bv > 1.0 ? 1.0 : Bv) * B0;
  const double rv = (rho ? rho[n] : 1.0) * rho0;
  const double ux = (u ? u[3 * n + 0] : 0.0) * u0;
  const double uy = (u ? u[3 * n + 1] : 0.0) * u0;
  const double uz = g.dim == 3 ? (u ? u[3 * n + 2] : 0.0) * u0 : 0.0;
  if (as_double) {
    if (solid_out) static_cast<double*>(solid_out)[id] = sv;
    if (rho_out) static_cast<double*>(rho_out)[id] = rv;
    if (u_out) {
      double* uo = static_cast<double*>(u_out);
      uo[3 * id + 0] = ux;
      uo[3 * id + 1] = uy;
      uo[3 * id + 2] = uz;
    }
  } else {
    if (solid_out) static_cast<float*>(solid_out)[id] = (float)sv;
    if (rho_out) static_cast<float*>(rho_out)[id] = (float)rv;
    if (u_out) {
      float* uo = static_cast<float*>(u_out);
      uo[3 * id + 0] = (float)ux;
      uo[3 * id + 1] = (float)uy;
      uo[3 * id + 2] = g.dim == 3 ? (float)uz : 0.0f;
    }
  }
}

cudaError_t launch_export_fields(const Geom& g, const Table& t, const double* rho, const double* u,
                                 int as_double, double B0, double rho0, double u0, void* solid_out,
                                 void* rho_out, void* u_out, cudaStream_t st) {
  const long long total =
      (long long)(g.L[0] - 2) * (g.L[1] - 2) * (g.dim == 3 ? g.L[2] - 2 : 1);
  if (total <= 0) return cudaSuccess;
  export_fields_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(
      g, t, rho, u, as_double, B0, rho0, u0, solid_out, rho_out, u_out);
  return cudaGetLastError();
}

}  // namespace lbmpsm
