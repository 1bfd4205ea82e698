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
    atomicAdd(p.pair_total, (unsigned long long)ncell);
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
  if (*p.pair_total > (unsigned long long)p.list_cap) {
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
  if (*p.pair_total > (unsigned long long)p.list_cap) return;
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

// calcSolidFraction (src/LBM_PSM_exchangeParticleData.cpp:116-169)
static __device__ double solid_fraction(int dim, int i, int j, int k, double xP, double yP,
                                        double zP, double rP_LB, double sqrt2half) {
  const int slicesPerDim = 10;
  const double sliceWidth = 1.0 / ((double)slicesPerDim);
  double fraction = 1.0 / ((double)(slicesPerDim * slicesPerDim));
  if (dim == 3) fraction = 1.0 / ((double)(slicesPerDim * slicesPerDim * slicesPerDim));
  const double dx = (double)i - xP;
  const double dy = (double)j - yP;
  const double dz = (double)k - zP;
  const double dist = dx * dx + dy * dy + dz * dz;
  const double rP = rP_LB + sqrt2half;
  if (dist > rP * rP) return 0.0;
  const double rM = rP_LB - sqrt2half;
  if (dist < rM * rM) return 1.0;
  const double rSq = rP_LB * rP_LB;
  double ax[10], ay[10], az[10];
  float fa[10], fb[10], fc[10];
  float amax = 0.f, bmax = 0.f, cmax = 0.f;
#pragma unroll
  for (int m = 0; m < 10; ++m) {
    const double delta = -0.5 + ((double)m + 0.5) * sliceWidth;
    const double dxi = dx + delta;
    ax[m] = dxi * dxi;
    const double dyi = dy + delta;
    ay[m] = dyi * dyi;
    const double dzi = dz + delta;
    az[m] = dzi * dzi;
    fa[m] = (float)ax[m];
    fb[m] = (float)ay[m];
    fc[m] = (float)az[m];
    amax = fmaxf(amax, fa[m]);
    bmax = fmaxf(bmax, fb[m]);
    cmax = fmaxf(cmax, fc[m]);
  }
  const float R = (float)rSq;
  int n = 0;
  if (dim == 2) {
    const float margin = 1.52587890625e-05f * fmaxf(R, amax + bmax);  // 2^-16
    for (int a = 0; a < 10; ++a) {
#pragma unroll
      for (int b = 0; b < 10; ++b) {
        const float d = (fa[a] + fb[b]) - R;
        if (d < -margin)
          ++n;
        else if (d <= margin && ax[a] + ay[b] < rSq)
          ++n;
      }
    }
  } else {
    const float margin = 1.52587890625e-05f * fmaxf(R, amax + bmax + cmax);
    for (int a = 0; a < 10; ++a) {
      for (int b = 0; b < 10; ++b) {
        const float s = fa[a] + fb[b];
#pragma unroll
        for (int c = 0; c < 10; ++c) {
          const float d = (s + fc[c]) - R;
          if (d < -margin)
            ++n;
          else if (d <= margin && ax[a] + ay[b] + az[c] < rSq)
            ++n;
        }
      }
    }
  }
  return fraction * ((double)n);
}

// setParticleOnLattice / setToZero on a register copy of one node's slots
struct NodeSlots {
  int id[2];
  double eps[2];
  double us[6];
};

static __device__ __forceinline__ void set_particle(NodeSlots& s, int pID, const double* uP,
                                                    double eps) {
  int slot = -1;
  if (s.id[0] == pID)
    slot = 0;
  else if (s.id[1] == pID)
    slot = 1;
  else if (pID != s.id[0] && pID != s.id[1] && s.id[0] == 0)
    slot = 0;
  else if (pID != s.id[0] && pID != s.id[1] && s.id[1] == 0)
    slot = 1;
  if (slot < 0) return;  // a third particle on the node is dropped
  s.id[slot] = pID;
  s.eps[slot] = eps;
  s.us[3 * slot + 0] = uP[0];
  s.us[3 * slot + 1] = uP[1];
  s.us[3 * slot + 2] = uP[2];
}

static __device__ __forceinline__ void set_to_zero(NodeSlots& s, int pID) {
  int slot = -1;
  if (s.id[0] == pID)
    slot = 0;
  else if (s.id[1] == pID)
    slot = 1;
  if (slot < 0) return;
  s.id[slot] = 0;
  s.eps[slot] = 0.0;
  s.us[3 * slot + 0] = 0.0;
  s.us[3 * slot + 1] = 0.0;
  s.us[3 * slot + 2] = 0.0;
}

__global__ void node_apply_kernel(MapParams p) {
  const int c = blockIdx.x;
  const int cnt = p.cell_count[c];
  if (cnt == 0) return;
  if (*p.pair_total > (unsigned long long)p.list_cap) return;
  const Geom& g = p.g;
  const int cx = c % p.C[0];
  const int cy = (c / p.C[0]) % p.C[1];
  const int cz = c / (p.C[0] * p.C[1]);
  const int sx = cx * p.cb[0] + threadIdx.x;
  const int sy = cy * p.cb[1] + threadIdx.y;
  const int sz = cz * p.cb[2] + threadIdx.z;
  if (sx >= g.S[0] || sy >= g.S[1] || sz >= g.S[2]) return;
  const long long n = ((long long)sz * g.S[1] + sy) * g.S[0] + sx;
  const int hi = sx + g.off[0], hj = sy + g.off[1], hk = sz + g.off[2];
  const int* lst = p.list + p.cell_off[c];
  NodeSlots s;
  bool loaded = false;
  for (int t = 0; t < cnt; ++t) {
    const Img& im = p.img[lst[t]];
    if (sx < im.lo[0] || sx >= im.hi[0] || sy < im.lo[1] || sy >= im.hi[1] || sz < im.lo[2] ||
        sz >= im.hi[2])
      continue;
    if (!loaded) {
      const int2 id = p.tab.ids[n];
      const double2 e = p.tab.eps[n];
      s.id[0] = id.x;
      s.id[1] = id.y;
      s.eps[0] = e.x;
      s.eps[1] = e.y;
      for (int k = 0; k < 6; ++k) s.us[k] = p.tab.us[6 * n + k];
      loaded = true;
    }
    const int tag = im.tag;
    const double sf = solid_fraction(g.dim, hi, hj, hk, im.xl[0], im.xl[1], im.xl[2], im.r,
                                     p.sqrt2half);
    int id_old = 0;
    double sf_old = 0.0;
    if (tag == s.id[0]) {
      id_old = s.id[0];
      sf_old = s.eps[0];
    } else if (tag == s.id[1]) {
      id_old = s.id[1];
      sf_old = s.eps[1];
    }
    const int decFlag = (sf > 0.00001) + 2 * (sf_old > 0.00001);
    const double dx = (double)hi - im.xl[0];
    const double dy = (double)hj - im.xl[1];
    const double dz = (double)hk - im.xl[2];
    double uNode[3];
    uNode[0] = im.uT[0] + im.om[1] * dz - im.om[2] * dy;
    uNode[1] = im.uT[1] + im.om[2] * dx - im.om[0] * dz;
    uNode[2] = im.uT[2] + im.om[0] * dy - im.om[1] * dx;
    switch (decFlag) {
      case 0:
        set_to_zero(s, tag);
        break;
      case 1:
        set_particle(s, tag, uNode, sf);
        break;
      case 2:
        if (id_old == tag) set_to_zero(s, tag);
        break;
      case 3:
        if (sf > sf_old || id_old == tag) set_particle(s, tag, uNode, sf);
        break;
    }
  }
  if (!loaded) return;
  p.tab.ids[n] = make_int2(s.id[0], s.id[1]);
  p.tab.eps[n] = make_double2(s.eps[0], s.eps[1]);
  for (int k = 0; k < 6; ++k) p.tab.us[6 * n + k] = s.us[k];
  p.tab.flag[n] = (uint8_t)((s.id[0] > 0 ? 1 : 0) | (s.id[1] > 0 ? 2 : 0));
  if (p.write32) {
    p.tab.rec32[2 * n] = make_float4((float)s.eps[0], (float)s.us[0], (float)s.us[1], (float)s.us[2]);
    p.tab.rec32[2 * n + 1] =
        make_float4((float)s.eps[1], (float)s.us[3], (float)s.us[4], (float)s.us[5]);
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
  dim3 block(p.cb[0], p.cb[1], p.cb[2]);
  node_apply_kernel<<<ncells, block, 0, st>>>(p);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ reduce
constexpr int RED_THREADS = 256;

__global__ void __launch_bounds__(RED_THREADS) reduce_kernel(ReduceParams p) {
  const int ip = blockIdx.x;
  const Geom& g = p.g;
  const int tag = p.tag[ip];
  const double r = p.radius[ip] / p.dx;
  double xl[3];
  int lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    xl[d] = local_centre(p.x[3 * ip + d], p.origin[d], p.dx);
    int a = (int)(xl[d] - r) - 2;
    int b = (int)(xl[d] + r) + 2;
    if (d < 2 || g.dim == 3) {
      a = clampi(a, 1, g.L[d] - 1);
      b = clampi(b, 1, g.L[d] - 1);
      if (d == 2) {
        if (a < 0) a = 0;
        if (b < 1) b = 1;
      }
    } else {
      // fmax(fmin(fmax(z, 1), nz - 1), slot) with nz = 1 in 2-D
      a = a < 1 ? 1 : a;
      a = a > g.L[2] - 1 ? g.L[2] - 1 : a;
      a = a < 0 ? 0 : a;
      b = b < 1 ? 1 : b;
      b = b > g.L[2] - 1 ? g.L[2] - 1 : b;
      b = b < 1 ? 1 : b;
    }
    lo[d] = a;
    hi[d] = b;
  }
  const int wx = hi[0] - lo[0], wy = hi[1] - lo[1], wz = hi[2] - lo[2];
  double acc[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) acc[k] = 0.0;
  if (wx > 0 && wy > 0 && wz > 0) {
    const long long total = (long long)wx * wy * wz;
    const double ff = p.forceFactor, tf = p.torqueFactor;
    for (long long t = threadIdx.x; t < total; t += RED_THREADS) {
      const int k = lo[2] + (int)(t % wz);
      const int j = lo[1] + (int)((t / wz) % wy);
      const int i = lo[0] + (int)(t / ((long long)wz * wy));
      const int sx = i - g.off[0], sy = j - g.off[1], sz = k - g.off[2];
      const long long n = ((long long)sz * g.S[1] + sy) * g.S[0] + sx;
      const int2 id = p.tab.ids[n];
      int slot;
      if (tag == id.x)
        slot = 0;
      else if (tag == id.y)
        slot = 1;
      else
        continue;
      double F0, F1, F2;
      if (p.nodeF_is_double) {
        const double* nf = static_cast<const double*>(p.tab.nodeF) + 6 * n + 3 * slot;
        F0 = nf[0];
        F1 = nf[1];
        F2 = nf[2];
      } else {
        const float* nf = static_cast<const float*>(p.tab.nodeF) + 6 * n + 3 * slot;
        F0 = nf[0];
        F1 = nf[1];
        F2 = nf[2];
      }
      acc[0] += F0 * ff;
      acc[1] += F1 * ff;
      acc[2] += F2 * ff;
      const double dx = (double)i - xl[0];
      const double dy = (double)j - xl[1];
      const double dz = (double)k - xl[2];
      acc[3] += (dy * F2 - dz * F1) * tf;
      acc[4] += (dz * F0 - dx * F2) * tf;
      acc[5] += (dx * F1 - dy * F0) * tf;
      acc[6] += 0.5 * (dx * F0 + dx * F0) * tf;
      acc[7] += 0.5 * (dy * F1 + dy * F1) * tf;
      acc[8] += 0.5 * (dz * F2 + dz * F2) * tf;
      acc[9] += 0.5 * (dy * F0 + dx * F1) * tf;
      acc[10] += 0.5 * (dz * F0 + dx * F2) * tf;
      acc[11] += 0.5 * (dz * F1 + dy * F2) * tf;
    }
  }
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
    double s = 0.0;
    for (int w = 0; w < RED_THREADS / 32; ++w) s += part[w][k];
    if (k < 3)
      p.fh[3 * ip + k] = s;
    else if (k < 6)
      p.th[3 * ip + (k - 3)] = s;
    else
      p.S[6 * ip + (k - 6)] = -s;
  }
}

cudaError_t launch_reduce(const ReduceParams& p, cudaStream_t st) {
  if (p.n <= 0) return cudaSuccess;
  reduce_kernel<<<p.n, RED_THREADS, 0, st>>>(p);
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
    const long long n = ((long long)sz * g.S[1] + sy) * g.S[0] + sx;
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
  const long long n = ((long long)sz * g.S[1] + sy) * g.S[0] + sx;
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
