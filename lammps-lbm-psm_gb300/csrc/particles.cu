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

__global__ void img_prep_kernel(MapParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const Geom& g = p.g;
  Img im;
  im.tag = p.tag[i];
  const double r = p.radius[i] / p.dx;
  im.r = r;
  bool valid = true;
  for (int d = 0; d < 3; ++d) {
    const double xl = local_centre(p.x[3 * i + d], p.origin[d], p.dx);
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
    im.lo[d] = slo;
    im.hi[d] = shi;
    if (slo >= shi) valid = false;
    im.uT[d] = p.v[3 * i + d] / p.Uc * p.u_lb;
    im.om[d] = p.omega[3 * i + d] * p.tc * p.dt_d;
  }
  im.valid = valid;
  {
    const double rP = r + p.sqrt2half;
    const double rM = r - p.sqrt2half;
    im.rP2 = rP * rP;
    im.rM2 = rM * rM;
    im.rSq = r * r;
    im.rP2f = (float)im.rP2;
    im.rM2f = (float)im.rM2;
    im.rSqf = (float)im.rSq;
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
    for (int d = 0; d < 3; ++d) {
      if (__double_as_longlong(im.om[d]) != 0ll) plain = false;
      if (__double_as_longlong(im.uT[d]) == (long long)0x8000000000000000ull) plain = false;
    }
    im.has_spin = plain ? 0 : 1;
  }
  im.sf_off = 0;
  for (int d = 0; d < 3; ++d) im.box[d] = valid ? im.hi[d] - im.lo[d] : 0;
  if (valid) {
    const unsigned long long vol = (unsigned long long)im.box[0] * im.box[1] * im.box[2];
    im.sf_off = (long long)atomicAdd(&p.pair_total[1], vol);
  }
  long long ncell = 0;
  if (valid) {
    for (int d = 0; d < 3; ++d) {
      im.clo[d] = im.lo[d] / p.cb[d];
      im.chi[d] = (im.hi[d] - 1) / p.cb[d];
    }
    ncell = (long long)(im.chi[0] - im.clo[0] + 1) * (im.chi[1] - im.clo[1] + 1) *
            (im.chi[2] - im.clo[2] + 1);
    for (int cz = im.clo[2]; cz <= im.chi[2]; ++cz)
      for (int cy = im.clo[1]; cy <= im.chi[1]; ++cy)
        for (int cx = im.clo[0]; cx <= im.chi[0]; ++cx)
          atomicAdd(&p.cell_count[(cz * p.C[1] + cy) * p.C[0] + cx], 1);
    atomicAdd(&p.pair_total[0], (unsigned long long)ncell);
  } else {
    for (int d = 0; d < 3; ++d) im.clo[d] = 0, im.chi[d] = -1;
  }
  p.img[i] = im;
}

// Exclusive scan of the cell counts, one block of 1024 threads.
__global__ void cell_scan_kernel(const int* __restrict__ count, int* __restrict__ off,
                                 int ncells) {
  __shared__ long long part[1024];
  const int t = threadIdx.x;
  const int chunk = (ncells + 1023) / 1024;
  const int b = t * chunk, e = min(ncells, b + chunk);
  long long s = 0;
  for (int c = b; c < e; ++c) s += count[c];
  part[t] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    long long v = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  long long run = part[t] - s;  // exclusive prefix of this chunk
  for (int c = b; c < e; ++c) {
    off[c] = (int)run;
    run += count[c];
  }
}

__global__ void img_fill_kernel(MapParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  if (p.pair_total[0] > (unsigned long long)p.list_cap ||
      p.pair_total[1] > (unsigned long long)p.sf_cap) {
    if (i == 0) atomicOr(p.status, STATUS_LIST_OVERFLOW);
    return;
  }
  const Img& im = p.img[i];
  if (!im.valid) return;
  for (int cz = im.clo[2]; cz <= im.chi[2]; ++cz)
    for (int cy = im.clo[1]; cy <= im.chi[1]; ++cy)
      for (int cx = im.clo[0]; cx <= im.chi[0]; ++cx) {
        const int c = (cz * p.C[1] + cy) * p.C[0] + cx;
        const int pos = atomicAdd(&p.cell_fill[c], 1);
        p.list[(long long)p.cell_off[c] + pos] = i;
      }
}

__global__ void cell_sort_kernel(MapParams p, int ncells) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  if (p.pair_total[0] > (unsigned long long)p.list_cap) return;
  int* a = p.list + p.cell_off[c];
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
}

// calcSolidFraction (src/LBM_PSM_exchangeParticleData.cpp:116-169): the
// sub-cell count evaluated exactly in FP64 with the reference's expressions,
// split over the 8 lanes of a group (lane `sub` takes the (a, b) rows sub,
// sub+8, ...).  All 32 lanes of the warp must call it (shuffles); lanes of
// groups without work pass valid = false.  Used whenever an FP32 decision
// cannot be proven equal to the reference's.
static __device__ int subcell_count_exact_group8(bool valid, int dim, double dx, double dy,
                                                 double dz, double rP_LB, int sub) {
  int n = 0;
  if (valid) {
    const double sliceWidth = 1.0 / ((double)10);
    const double rSq = rP_LB * rP_LB;
    double az[10];
#pragma unroll
    for (int c = 0; c < 10; ++c) {
      const double delta = -0.5 + ((double)c + 0.5) * sliceWidth;
      const double dzi = dz + delta;
      az[c] = dzi * dzi;
    }
    for (int r = sub; r < 100; r += 8) {
      const int a = r / 10, b = r % 10;
      const double da = dx + (-0.5 + ((double)a + 0.5) * sliceWidth);
      const double db = dy + (-0.5 + ((double)b + 0.5) * sliceWidth);
      const double ax = da * da, ay = db * db;
      if (dim == 2) {
        if (ax + ay < rSq) ++n;
      } else {
#pragma unroll
        for (int c = 0; c < 10; ++c)
          if (ax + ay + az[c] < rSq) ++n;
      }
    }
  }
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  return n;
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

constexpr int SF_THREADS = 256;
constexpr int SF_ROUND = 2048;  // box nodes classified per round (queue capacity)
constexpr int SF_WBUF = 64;     // per-warp buffer of crossing rows

static __device__ __forceinline__ float sub_offset(int k) {
  return -0.45f + 0.1f * small_int_to_float(k);  // within 1.7u of the reference's delta_k
}

// Phase 1 of the map: solid-fraction codes of every node of every image box
// (independent of image order).  One block per image.  Box nodes are
// classified per thread; shell nodes go to a shared-memory queue and are then
// counted one per lane: every lane walks its node's 100 rows of 10 sub-cells
// in a warp-uniform loop, counting rows wholly inside in registers, and pushes
// rows that cross the surface into a per-warp buffer that is drained 32 rows
// at a time, one row per lane (so no lane idles on another's crossing row).
// Nodes where any sub-cell sum falls inside the FP32 margin are recounted
// exactly in FP64.
__global__ void __launch_bounds__(SF_THREADS) sf_kernel(MapParams p) {
  const Img& im = p.img[blockIdx.x];
  if (!im.valid) return;
  if (p.pair_total[0] > (unsigned long long)p.list_cap ||
      p.pair_total[1] > (unsigned long long)p.sf_cap)
    return;
  const Geom& g = p.g;
  const int wx = im.box[0], wy = im.box[1], wz = im.box[2];
  const int vol = wx * wy * wz;
  unsigned short* code = p.sfcode + im.sf_off;
  constexpr int NW = SF_THREADS / 32;
  __shared__ int queue[SF_ROUND];
  __shared__ int exact_list[SF_ROUND];
  __shared__ float buf_s[NW][SF_WBUF];
  __shared__ int buf_o[NW][SF_WBUF];
  __shared__ float np_dc[NW][32], np_lo[NW][32], np_hi[NW][32];
  __shared__ int wcnt[NW][32], wamb[NW][32];
  __shared__ int qn, nex;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float u = 5.9604644775390625e-08f;  // 2^-24
  const FastDiv fx = make_fastdiv((unsigned)wx), fy = make_fastdiv((unsigned)wy);
  for (int base = 0; base < vol; base += SF_ROUND) {
    if (threadIdx.x == 0) {
      qn = 0;
      nex = 0;
    }
    __syncthreads();
    const int end = min(vol, base + SF_ROUND);
    for (int li = base + threadIdx.x; li < end; li += SF_THREADS) {
      const int q1 = (int)fast_div((unsigned)li, fx);
      const int q2 = (int)fast_div((unsigned)q1, fy);
      const int sx = im.lo[0] + li - q1 * wx;
      const int sy = im.lo[1] + q1 - q2 * wy;
      const int sz = im.lo[2] + q2;
      float dxf, dyf, dzf;
      const int c = classify_node(sx + g.off[0], sy + g.off[1], sz + g.off[2], im, dxf, dyf, dzf);
      if (c >= 0)
        code[li] = (unsigned short)c;
      else
        queue[atomicAdd(&qn, 1)] = li;
    }
    __syncthreads();
    const int nq = qn;
    for (int e0 = warp * 32; e0 < nq; e0 += SF_THREADS) {
      const int e = e0 + lane;
      const bool valid = e < nq;
      const int li = valid ? queue[e] : queue[e0];
      const int q1 = (int)fast_div((unsigned)li, fx);
      const int q2 = (int)fast_div((unsigned)q1, fy);
      const float dxf = small_int_to_float(im.lo[0] + li - q1 * wx + g.off[0] - im.xi[0]) - im.xf[0];
      const float dyf = small_int_to_float(im.lo[1] + q1 - q2 * wy + g.off[1] - im.xi[1]) - im.xf[1];
      const float dzf = small_int_to_float(im.lo[2] + q2 + g.off[2] - im.xi[2]) - im.xf[2];
      // axis order: outer a, middle b, inner c along the smallest |d|
      float da = dxf, db = dyf, dc = dzf;
      if (g.dim == 3) {
        const float ax = fabsf(dxf), ay = fabsf(dyf), az = fabsf(dzf);
        if (ax <= ay && ax <= az) {
          da = dyf; db = dzf; dc = dxf;
        } else if (ay <= ax && ay <= az) {
          da = dxf; db = dzf; dc = dyf;
        }
      }
      const float Ea = fabsf(da) + 2.0f, Eb = fabsf(db) + 2.0f, Ec = fabsf(dc) + 2.0f;
      const float Emax = g.dim == 3 ? Ea * Ea + Eb * Eb + Ec * Ec : Ea * Ea + Eb * Eb;
      const float M = 16.0f * u * (Emax + im.rSqf);
      const float lo = im.rSqf - M, hi = im.rSqf + M;
      int n = 0, amb = 0;
      if (g.dim == 2) {
        for (int a = 0; a < 10; ++a) {
          const float ta = da + sub_offset(a);
          const float sa = ta * ta;
#pragma unroll
          for (int b = 0; b < 10; ++b) {
            const float tb = db + (float)(-0.5 + ((double)b + 0.5) * 0.1);
            const float t = sa + tb * tb;
            n += (t < lo);
            amb += (t >= lo) & (t <= hi);
          }
        }
      } else {
        float cmin = 3.4e38f, cmax = 0.0f;
#pragma unroll
        for (int k = 0; k < 10; ++k) {
          const float t = dc + (float)(-0.5 + ((double)k + 0.5) * 0.1);
          cmin = fminf(cmin, t * t);
          cmax = fmaxf(cmax, t * t);
        }
        np_dc[warp][lane] = dc;
        np_lo[warp][lane] = lo;
        np_hi[warp][lane] = hi;
        wcnt[warp][lane] = 0;
        wamb[warp][lane] = 0;
        __syncwarp();
        int wcount = 0;
        for (int a = 0; a < 10; ++a) {
          const float ta = da + sub_offset(a);
          const float sa = ta * ta;
          for (int b = 0; b < 10; ++b) {
            const float tb = db + sub_offset(b);
            const float sv = sa + tb * tb;
            const bool inside = sv + cmax < lo;
            const bool cross = valid && !inside && !(sv + cmin > hi);
            n += inside ? 10 : 0;
            const unsigned m = __ballot_sync(0xffffffffu, cross);
            if (cross) {
              const int pos = wcount + __popc(m & ((1u << lane) - 1u));
              buf_s[warp][pos] = sv;
              buf_o[warp][pos] = lane;
            }
            wcount += __popc(m);
            if (wcount >= 32) {
              __syncwarp();
              const int k = wcount - 32 + lane;
              const float sk = buf_s[warp][k];
              const int ow = buf_o[warp][k];
              const float dco = np_dc[warp][ow], loo = np_lo[warp][ow], hio = np_hi[warp][ow];
              int nn = 0, na = 0;
#pragma unroll
              for (int cc = 0; cc < 10; ++cc) {
                const float tc = dco + (float)(-0.5 + ((double)cc + 0.5) * 0.1);
                const float t = sk + tc * tc;
                nn += (t < loo);
                na += (t >= loo) & (t <= hio);
              }
              if (nn) atomicAdd(&wcnt[warp][ow], nn);
              if (na) atomicAdd(&wamb[warp][ow], na);
              wcount -= 32;
              __syncwarp();
            }
          }
        }
        __syncwarp();
        if (lane < wcount) {
          const float sk = buf_s[warp][lane];
          const int ow = buf_o[warp][lane];
          const float dco = np_dc[warp][ow], loo = np_lo[warp][ow], hio = np_hi[warp][ow];
          int nn = 0, na = 0;
#pragma unroll
          for (int cc = 0; cc < 10; ++cc) {
            const float tc = dco + (float)(-0.5 + ((double)cc + 0.5) * 0.1);
            const float t = sk + tc * tc;
            nn += (t < loo);
            na += (t >= loo) & (t <= hio);
          }
          if (nn) atomicAdd(&wcnt[warp][ow], nn);
          if (na) atomicAdd(&wamb[warp][ow], na);
        }
        __syncwarp();
        n += wcnt[warp][lane];
        amb += wamb[warp][lane];
        __syncwarp();
      }
      if (valid) {
        if (amb == 0)
          code[li] = (unsigned short)n;
        else
          exact_list[atomicAdd(&nex, 1)] = li;
      }
    }
    __syncthreads();
    // exact FP64 recount of the ambiguous nodes, four per warp
    const int ne = nex;
    const int grp = lane >> 3, sub = lane & 7;
    for (int e0 = warp * 4; e0 < ne; e0 += NW * 4) {
      const int e = e0 + grp;
      const bool valid = e < ne;
      const int li = valid ? exact_list[e] : 0;
      const int q1 = (int)fast_div((unsigned)li, fx);
      const int q2 = (int)fast_div((unsigned)q1, fy);
      const int hi = im.lo[0] + li - q1 * wx + g.off[0];
      const int hj = im.lo[1] + q1 - q2 * wy + g.off[1];
      const int hk = im.lo[2] + q2 + g.off[2];
      const int nc = subcell_count_exact_group8(valid, g.dim, (double)hi - im.xl[0],
                                                (double)hj - im.xl[1], (double)hk - im.xl[2],
                                                im.r, sub);
      if (valid && sub == 0) code[li] = (unsigned short)nc;
    }
    __syncthreads();
  }
}

// Phase 2 of the map: per node, the images whose boxes contain it, in image
// order, through the 4-way update of setParticlesOnLattice
// (src/LBM_PSM_exchangeParticleData.cpp:69-106) on the two-slot table
// (setParticleOnLattice / setToZero, src/LBM_PSM_lattice.cpp:257-324).
// The table is written back only where it changed.
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
  const int hi = sx + g.off[0], hj = sy + g.off[1], hk = sz + g.off[2];
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
    bool same = !slot_dirty[slot] && id[slot] == tag &&
                __double_as_longlong(eps[slot]) == __double_as_longlong(sf);
    if (same) {
      const double* cur = p.tab.us + 6 * n + 3 * slot;
      same = __double_as_longlong(cur[0]) == __double_as_longlong(u0) &&
             __double_as_longlong(cur[1]) == __double_as_longlong(u1) &&
             __double_as_longlong(cur[2]) == __double_as_longlong(u2);
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

cudaError_t launch_map(const MapParams& p, cudaStream_t st) {
  if (p.n <= 0) return cudaSuccess;
  const int ncells = p.C[0] * p.C[1] * p.C[2];
  const int tb = 128;
  img_prep_kernel<<<(p.n + tb - 1) / tb, tb, 0, st>>>(p);
  cell_scan_kernel<<<1, 1024, 0, st>>>(p.cell_count, p.cell_off, ncells);
  img_fill_kernel<<<(p.n + tb - 1) / tb, tb, 0, st>>>(p);
  cell_sort_kernel<<<(ncells + 255) / 256, 256, 0, st>>>(p, ncells);
  sf_kernel<<<p.n, SF_THREADS, 0, st>>>(p);
  dim3 block(p.cb[0], p.cb[1], p.cb[2]);
  dim3 cells((unsigned)p.C[0], (unsigned)p.C[1], (unsigned)p.C[2]);
  node_apply_kernel<<<cells, block, 0, st>>>(p);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ reduce
constexpr int RED_THREADS = 256;

// Box of one image clamped to interior nodes (src/LBM_PSM_exchangeParticleData.cpp:188-195).
struct RedBox {
  double xl[3];
  int lo[3], hi[3];
};

static __device__ __forceinline__ RedBox reduce_box(const ReduceParams& p, int ip) {
  const Geom& g = p.g;
  RedBox b;
  const double r = p.radius[ip] / p.dx;
  for (int d = 0; d < 3; ++d) {
    b.xl[d] = local_centre(p.x[3 * ip + d], p.origin[d], p.dx);
    int a = (int)(b.xl[d] - r) - 2;
    int c = (int)(b.xl[d] + r) + 2;
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
    b.lo[d] = a;
    b.hi[d] = c;
  }
  return b;
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
    if (k < 3)
      p.fh[3 * ip + k] = sum;
    else if (k < 6)
      p.th[3 * ip + (k - 3)] = sum;
    else
      p.S[6 * ip + (k - 6)] = -sum;
  }
}

// FP64 node forces (FP64 storage): the reference's per-node terms in FP64.
__global__ void __launch_bounds__(RED_THREADS) reduce_f64_kernel(ReduceParams p) {
  const int ip = blockIdx.x;
  const Geom& g = p.g;
  const int tag = p.tag[ip];
  const RedBox bx = reduce_box(p, ip);
  const int wx = bx.hi[0] - bx.lo[0], wy = bx.hi[1] - bx.lo[1], wz = bx.hi[2] - bx.lo[2];
  double acc[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) acc[k] = 0.0;
  if (wx > 0 && wy > 0 && wz > 0) {
    const long long total = (long long)wx * wy * wz;
    const double ff = p.forceFactor, tf = p.torqueFactor;
    const double* nodeF = static_cast<const double*>(p.tab.nodeF);
    const FastDiv fz = make_fastdiv((unsigned)wz), fy = make_fastdiv((unsigned)wy);
    for (long long t = threadIdx.x; t < total; t += RED_THREADS) {
      const int q1 = (int)fast_div((unsigned)t, fz);
      const int q2 = (int)fast_div((unsigned)q1, fy);
      const int k = bx.lo[2] + (int)t - q1 * wz;
      const int j = bx.lo[1] + q1 - q2 * wy;
      const int i = bx.lo[0] + q2;
      const long long n = node_index(g, i - g.off[0], j - g.off[1], k - g.off[2]);
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
}

// Error-free transformation: a + b = s + e exactly (Knuth's TwoSum; no
// contraction or reassociation under -fmad=false).
static __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// FP32 node forces (FP32 / FP16 storage): per-node terms in FP32 (the node
// forces carry FP32 precision), accumulated per particle in double-float
// (hi + lo pairs combined with TwoSum, ~48-bit significand) on the FP32 pipe,
// then the per-warp results summed in FP64.  (FP64 arithmetic runs at 1/64 of
// the FP32 rate on this GPU.)
__global__ void __launch_bounds__(RED_THREADS) reduce_f32_kernel(ReduceParams p) {
  const int ip = blockIdx.x;
  const Geom& g = p.g;
  const int tag = p.tag[ip];
  const RedBox bx = reduce_box(p, ip);
  const int wx = bx.hi[0] - bx.lo[0], wy = bx.hi[1] - bx.lo[1], wz = bx.hi[2] - bx.lo[2];
  float hi[12], lo[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) hi[k] = lo[k] = 0.0f;
  if (wx > 0 && wy > 0 && wz > 0) {
    int xi[3];
    float xf[3];
    for (int d = 0; d < 3; ++d) {
      const double fl = fabs(bx.xl[d]) < 1.0e9 ? floor(bx.xl[d]) : 0.0;
      xi[d] = (int)fl;
      xf[d] = (float)(bx.xl[d] - fl);
    }
    const int total = wx * wy * wz;
    const float* nodeF = static_cast<const float*>(p.tab.nodeF);
    const FastDiv fz = make_fastdiv((unsigned)wz), fy = make_fastdiv((unsigned)wy);
    for (int t = threadIdx.x; t < total; t += RED_THREADS) {
      const int q1 = (int)fast_div((unsigned)t, fz);
      const int q2 = (int)fast_div((unsigned)q1, fy);
      const int k = bx.lo[2] + t - q1 * wz;
      const int j = bx.lo[1] + q1 - q2 * wy;
      const int i = bx.lo[0] + q2;
      const long long n = node_index(g, i - g.off[0], j - g.off[1], k - g.off[2]);
      const int2 id = p.tab.ids[n];
      int slot;
      if (tag == id.x)
        slot = 0;
      else if (tag == id.y)
        slot = 1;
      else
        continue;
      const float* nf = nodeF + 6 * n + 3 * slot;
      const float F0 = nf[0], F1 = nf[1], F2 = nf[2];
      const float dx = small_int_to_float(i - xi[0]) - xf[0];
      const float dy = small_int_to_float(j - xi[1]) - xf[1];
      const float dz = small_int_to_float(k - xi[2]) - xf[2];
      const float term[12] = {F0,
                              F1,
                              F2,
                              dy * F2 - dz * F1,
                              dz * F0 - dx * F2,
                              dx * F1 - dy * F0,
                              dx * F0,
                              dy * F1,
                              dz * F2,
                              0.5f * (dy * F0 + dx * F1),
                              0.5f * (dz * F0 + dx * F2),
                              0.5f * (dz * F1 + dy * F2)};
#pragma unroll
      for (int q = 0; q < 12; ++q) {
        float sv, e;
        two_sum(hi[q], term[q], sv, e);
        hi[q] = sv;
        lo[q] += e;
      }
    }
  }
  // fixed-order double-float butterfly within the warp
#pragma unroll
  for (int q = 0; q < 12; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float h2 = __shfl_xor_sync(0xffffffffu, hi[q], o);
      const float l2 = __shfl_xor_sync(0xffffffffu, lo[q], o);
      float sv, e;
      two_sum(hi[q], h2, sv, e);
      hi[q] = sv;
      lo[q] = lo[q] + l2 + e;
    }
  }
  __shared__ double part[RED_THREADS / 32][12];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int q = 0; q < 12; ++q) part[warp][q] = (double)hi[q] + (double)lo[q];
  __syncthreads();
  if (threadIdx.x < 12) {
    const int q = threadIdx.x;
    double sum = 0.0;
    for (int w = 0; w < RED_THREADS / 32; ++w) sum += part[w][q];
    if (q < 3)
      p.fh[3 * ip + q] = sum * p.forceFactor;
    else if (q < 6)
      p.th[3 * ip + (q - 3)] = sum * p.torqueFactor;
    else
      p.S[6 * ip + (q - 6)] = -(sum * p.torqueFactor);
  }
}

cudaError_t launch_reduce(const ReduceParams& p, cudaStream_t st) {
  if (p.n <= 0) return cudaSuccess;
  if (p.nodeF_is_double)
    reduce_f64_kernel<<<p.n, RED_THREADS, 0, st>>>(p);
  else
    reduce_f32_kernel<<<p.n, RED_THREADS, 0, st>>>(p);
  return cudaGetLastError();
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
    e = t.eps[n];
    for (int c = 0; c < 6; ++c) u[c] = t.us[6 * n + c];
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
  const double2 e = t.eps[n];
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
