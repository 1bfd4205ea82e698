// collide_lowp.cu -- FP32-collision paths of the fused collide / A-A stream
// kernel and the Zou-He face kernel.
//
// Populations are stored as deviations g_q = f_q - w_q*rho0 (rho0 = 1): in
// FP32 (LBMPSM_STORAGE_FP32) or in FP16 scaled by scale16
// (LBMPSM_STORAGE_FP16).  The collision runs in FP32 on the deviations, which
// keeps the small differences f - feq of a low-Mach flow well resolved; the
// algebra is the reference's (src/LBM_PSM_BGK_dynamics.h:40-114,
// src/LBM_PSM_dynamics.h:43-116) with the w_q*rho0 parts cancelled:
//   feq_q - w_q = w_q (drho + rho (3 e.u + 4.5 (e.u)^2 - 1.5 u.u)).
// Node forces of PSM nodes are written in FP32 and reduced per particle in
// FP64 (particles.cu).
#include <cuda_fp16.h>

#include "lbmpsm_internal.cuh"

namespace lbmpsm {

template <typename T>
struct Store;
template <>
struct Store<float> {
  __device__ __forceinline__ static float load(const float* p, float) { return *p; }
  __device__ __forceinline__ static void store(float* p, float v, float) { *p = v; }
};
template <>
struct Store<__half> {
  __device__ __forceinline__ static float load(const __half* p, float scale) {
    return __half2float(*p) * (1.0f / scale);
  }
  __device__ __forceinline__ static void store(__half* p, float v, float scale) {
    *p = __float2half_rn(v * scale);
  }
};

template <int cx, int cy, int cz>
__device__ __forceinline__ float edotf(float vx, float vy, float vz) {
  float s = 0.0f;
  if (cx) s += cx > 0 ? vx : -vx;
  if (cy) s += cy > 0 ? vy : -vy;
  if (cz) s += cz > 0 ? vz : -vz;
  return s;
}

struct PsmNodeF {
  bool has1, has2;
  float B1, B2, omB;   // omB = (1 - Btot) * omega
  float us1[3], us2[3];
  float q1, q2;        // 1.5 |us|^2
  float F1[3], F2[3];
};

// Guo forcing term (src/LBM_PSM_dynamics.h:102-116) in deviation form
template <class L, int q>
__device__ __forceinline__ float guo_f32(float ux, float uy, float uz, float eu, float gpref,
                                         float Fx, float Fy, float Fz) {
  constexpr int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
  const float w = (float)L::w(q);
  const float a = ((float)cx - ux) * Fx + ((float)cy - uy) * Fy + ((float)cz - uz) * Fz;
  const float eF = edotf<cx, cy, cz>(Fx, Fy, Fz);
  return gpref * w * (3.0f * a + 9.0f * eu * eF);
}

// PSM collision of direction q (src/LBM_PSM_BGK_dynamics.h:70-113)
template <class L, int q, bool FORCE>
__device__ __forceinline__ void collide_q_psm(float& gq, float drho, float rho, float ux,
                                              float uy, float uz, float usq15, float omo,
                                              float gpref, float Fx, float Fy, float Fz,
                                              PsmNodeF& sn) {
  constexpr int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
  const float w = (float)L::w(q);
  const float g = gq;
  const float eu = edotf<cx, cy, cz>(ux, uy, uz);
  const float geq = w * (drho + rho * (3.0f * eu + 4.5f * eu * eu - usq15));
  const float Fq = FORCE ? guo_f32<L, q>(ux, uy, uz, eu, gpref, Fx, Fy, Fz) : 0.0f;
  float sc1 = 0.0f, sc2 = 0.0f;
  if (sn.has1) {
    const float e1 = edotf<cx, cy, cz>(sn.us1[0], sn.us1[1], sn.us1[2]);
    const float gs = w * (drho + rho * (3.0f * e1 + 4.5f * e1 * e1 - sn.q1));
    sc1 = (gs - g) + omo * (g - geq);
  }
  if (sn.has2) {
    const float e2 = edotf<cx, cy, cz>(sn.us2[0], sn.us2[1], sn.us2[2]);
    const float gs = w * (drho + rho * (3.0f * e2 + 4.5f * e2 * e2 - sn.q2));
    sc2 = (gs - g) + omo * (g - geq);
  }
  gq = g + sn.omB * (geq - g) + sn.B1 * sc1 + sn.B2 * sc2 + Fq;
  if (sn.has1) {
    const float t = -sn.B1 * sc1;
    if (cx) sn.F1[0] += cx > 0 ? t : -t;
    if (cy) sn.F1[1] += cy > 0 ? t : -t;
    if (cz) sn.F1[2] += cz > 0 ? t : -t;
  }
  if (sn.has2) {
    const float t = -sn.B2 * sc2;
    if (cx) sn.F2[0] += cx > 0 ? t : -t;
    if (cy) sn.F2[1] += cy > 0 ? t : -t;
    if (cz) sn.F2[2] += cz > 0 ? t : -t;
  }
}

template <class L, int q, bool FORCE>
struct UnrollPsm {
  __device__ __forceinline__ static void run(float* g, float drho, float rho, float ux, float uy,
                                             float uz, float usq15, float omo, float gpref,
                                             float Fx, float Fy, float Fz, PsmNodeF& sn) {
    collide_q_psm<L, q, FORCE>(g[q], drho, rho, ux, uy, uz, usq15, omo, gpref, Fx, Fy, Fz, sn);
    UnrollPsm<L, q + 1, FORCE>::run(g, drho, rho, ux, uy, uz, usq15, omo, gpref, Fx, Fy, Fz, sn);
  }
};
template <class L, bool FORCE>
struct UnrollPsm<L, L::Q, FORCE> {
  __device__ __forceinline__ static void run(float*, float, float, float, float, float, float,
                                             float, float, float, float, float, PsmNodeF&) {}
};

// plain BGK collision of every direction with the Guo term
template <class L, int q, bool FORCE>
struct UnrollFluid {
  __device__ __forceinline__ static void run(float* g, float drho, float rho, float ux, float uy,
                                             float uz, float usq15, float omega, float gpref,
                                             float Fx, float Fy, float Fz) {
    constexpr int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    const float w = (float)L::w(q);
    const float eu = edotf<cx, cy, cz>(ux, uy, uz);
    const float geq = w * (drho + rho * (3.0f * eu + 4.5f * eu * eu - usq15));
    const float Fq = FORCE ? guo_f32<L, q>(ux, uy, uz, eu, gpref, Fx, Fy, Fz) : 0.0f;
    g[q] = g[q] + omega * (geq - g[q]) + Fq;
    UnrollFluid<L, q + 1, FORCE>::run(g, drho, rho, ux, uy, uz, usq15, omega, gpref, Fx, Fy, Fz);
  }
};
template <class L, bool FORCE>
struct UnrollFluid<L, L::Q, FORCE> {
  __device__ __forceinline__ static void run(float*, float, float, float, float, float, float,
                                             float, float, float, float, float) {}
};

// Collision of one node on its Q deviations f[], in place: macro values,
// optional macro store, then either the plain BGK update (fluid node) or the
// PSM solid operator with node forces.  flag / r1 / r2 are the node's table
// entries, loaded by the caller.
template <class L, bool FORCE>
__device__ __forceinline__ void collide_node_lowp(float (&f)[L::Q], const CollideParams& p,
                                                  long long n, uint8_t flag, float4 r1,
                                                  float4 r2) {
  constexpr int Q = L::Q;
  float drho = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    drho += f[q];
    if (cx) jx += cx > 0 ? f[q] : -f[q];
    if (cy) jy += cy > 0 ? f[q] : -f[q];
    if (cz) jz += cz > 0 ? f[q] : -f[q];
  }
  const float Fx = p.F_f[0], Fy = p.F_f[1], Fz = p.F_f[2];
  if (FORCE) {
    jx += 0.5f * Fx;
    jy += 0.5f * Fy;
    jz += 0.5f * Fz;
  }
  const float rho = 1.0f + drho;
  const float inv = __frcp_rn(rho);
  const float ux = jx * inv, uy = jy * inv, uz = jz * inv;
  if (p.store_macro) {
    p.rho_out[n] = 1.0 + (double)drho;
    p.u_out[3 * n + 0] = ux;
    p.u_out[3 * n + 1] = uy;
    p.u_out[3 * n + 2] = uz;
  }
  const float usq15 = 1.5f * (ux * ux + uy * uy + uz * uz);
  const float omega = p.omega_f;
  if (flag == 0) {
    UnrollFluid<L, 0, FORCE>::run(f, drho, rho, ux, uy, uz, usq15, omega, p.gpref_f, Fx, Fy, Fz);
    return;
  }
  PsmNodeF sn;
  sn.has1 = (flag & 1) != 0;
  sn.has2 = (flag & 2) != 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) sn.F1[c] = sn.F2[c] = 0.0f;
  float B1 = sn.has1 ? r1.x : 0.0f;
  float B2 = sn.has2 ? r2.x : 0.0f;
  if (p.weighting == 1) {  // Noble-Torczynski weighting (opt-in)
    const float tm = p.tm_f;
    if (sn.has1) B1 = B1 * tm / ((1.0f - B1) + tm);
    if (sn.has2) B2 = B2 * tm / ((1.0f - B2) + tm);
  }
  float Bt = B1 + B2;
  if (Bt > 1.0f) {
    B1 = B1 / Bt;
    B2 = B2 / Bt;
    Bt = 1.0f;
  }
  sn.B1 = B1;
  sn.B2 = B2;
  sn.omB = (1.0f - Bt) * omega;
  sn.us1[0] = sn.has1 ? r1.y : 0.0f;
  sn.us1[1] = sn.has1 ? r1.z : 0.0f;
  sn.us1[2] = sn.has1 ? r1.w : 0.0f;
  sn.us2[0] = sn.has2 ? r2.y : 0.0f;
  sn.us2[1] = sn.has2 ? r2.z : 0.0f;
  sn.us2[2] = sn.has2 ? r2.w : 0.0f;
  sn.q1 = 1.5f * (sn.us1[0] * sn.us1[0] + sn.us1[1] * sn.us1[1] + sn.us1[2] * sn.us1[2]);
  sn.q2 = 1.5f * (sn.us2[0] * sn.us2[0] + sn.us2[1] * sn.us2[1] + sn.us2[2] * sn.us2[2]);
  UnrollPsm<L, 0, FORCE>::run(f, drho, rho, ux, uy, uz, usq15, p.omo_f, p.gpref_f, Fx, Fy, Fz, sn);
  float* nf = static_cast<float*>(p.tab.nodeF) + 6 * n;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    nf[c] = sn.F1[c];
    nf[3 + c] = sn.F2[c];
  }
}

// Direct variant: each thread gathers its node's populations from global
// memory (used when an x-row is longer than one staged block).
template <class L, typename T, bool ODD, bool FORCE>
__global__ void __launch_bounds__(128) collide_lowp_kernel(CollideParams p) {
  constexpr int Q = L::Q;
  const Geom& g = p.g;
  // blocks: (row, x-chunk) folded into blockIdx.x (rows can exceed the 65535 limit of y)
  const int xblocks = (g.S[0] + blockDim.x - 1) / blockDim.x;
  const int row = blockIdx.x / xblocks;
  const int sx = (blockIdx.x - row * xblocks) * blockDim.x + threadIdx.x;
  if (sx >= g.S[0]) return;
  const int sy = row % g.S[1];
  const int sz = row / g.S[1];
  const long long n = node_index(g, sx, sy, sz);
  const Nbr nb = make_nbr(g, sx, sy, sz);
  T* __restrict__ F = static_cast<T*>(p.f);
  const long long Np = g.Np;
  const float sc = p.scale16;
  float f[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    const bool ok = nbr_ok(nb, -cx, -cy, -cz);
    if (!ODD) {
      f[q] = ok ? Store<T>::load(F + q * Np + n, sc) : 0.0f;
    } else {
      const int o = nbr_off(nb, -cx, -cy, -cz);
      f[q] = ok ? Store<T>::load(F + L::opp(q) * Np + n + o, sc) : 0.0f;
    }
  }
  const uint8_t flag = p.tab.flag[n];
  float4 r1 = make_float4(0.f, 0.f, 0.f, 0.f), r2 = r1;
  if (flag) {
    r1 = p.tab.rec32[2 * n];
    r2 = p.tab.rec32[2 * n + 1];
  }
  collide_node_lowp<L, FORCE>(f, p, n, flag, r1, r2);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    if (!ODD) {
      Store<T>::store(F + L::opp(q) * Np + n, f[q], sc);
    } else {
      if (nbr_ok(nb, cx, cy, cz)) Store<T>::store(F + q * Np + n + nbr_off(nb, cx, cy, cz), f[q], sc);
    }
  }
}

// ------------------------------------------------------------- row staging
// Bulk asynchronous copies (cp.async.bulk, the 1-D form of the tensor memory
// accelerator path) between global memory and shared memory, completed on an
// mbarrier for loads and through a bulk group for stores.
__device__ __forceinline__ unsigned smem_addr(const void* ptr) {
  return static_cast<unsigned>(__cvta_generic_to_shared(ptr));
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred P1;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, P1;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(phase)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_load(unsigned dst, const void* src, unsigned bytes,
                                          unsigned bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void bulk_store(void* dst, unsigned src, unsigned bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

constexpr int STAGED_MAX_ROW = 256;      // nodes per x-row handled by one staged block
constexpr long long MBAR_SPIN_LIMIT = 1ll << 26;

// neighbour row (dy, dz) of row (sy, sz); false when it does not exist
__device__ __forceinline__ bool row_of(const Geom& g, int sy, int sz, int dy, int dz,
                                       long long& base) {
  int y = sy + dy, z = sz + dz;
  if (y < 0 || y >= g.S[1]) {
    if (!g.per[1]) return false;
    y = y < 0 ? y + g.S[1] : y - g.S[1];
  }
  if (z < 0 || z >= g.S[2]) {
    if (!g.per[2]) return false;
    z = z < 0 ? z + g.S[2] : z - g.S[2];
  }
  base = ((long long)z * g.S[1] + y) * g.P0;
  return true;
}

// bit (dy+1)*3 + (dz+1) set when row (sy+dy, sz+dz) exists
__device__ __forceinline__ unsigned row_mask(const Geom& g, int sy, int sz) {
  unsigned m = 0;
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz) {
      const int y = sy + dy, z = sz + dz;
      const bool oky = (y >= 0 && y < g.S[1]) || g.per[1];
      const bool okz = (z >= 0 && z < g.S[2]) || g.per[2];
      if (oky && okz) m |= 1u << ((dy + 1) * 3 + (dz + 1));
    }
  return m;
}
__host__ __device__ constexpr int row_bit(int dy, int dz) { return (dy + 1) * 3 + (dz + 1); }

// Staged variant: one block per x-row (sy, sz), one thread per node.  The Q
// population rows the step reads are pulled into shared memory with one bulk
// copy each, the x-shifts of streaming are applied as shared-memory index
// offsets, and the Q output rows are pushed back with one bulk copy each.
//   even step: own row, slot q in, slot opp(q) out;
//   odd step : row -e_q, slot opp(q) in -> row +e_q, slot q out.
// The A-A pattern makes each block the only reader and writer of the
// locations it moves, so blocks need no synchronisation between them.
template <class L, typename T, bool ODD, bool FORCE>
__global__ void __launch_bounds__(STAGED_MAX_ROW, 4) collide_staged_kernel(CollideParams p) {
  constexpr int Q = L::Q;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const Geom& g = p.g;
  const int P0 = g.P0;
  T* buf = reinterpret_cast<T*>(smem_raw);
  const unsigned bar = smem_addr(smem_raw + (size_t)Q * P0 * sizeof(T));
  const unsigned row_bytes = (unsigned)(P0 * sizeof(T));
  const int sy = blockIdx.x;
  const int sz = blockIdx.y;
  const long long own = ((long long)sz * g.S[1] + sy) * P0;
  T* __restrict__ F = static_cast<T*>(p.f);
  const long long Np = g.Np;
  const float sc = p.scale16;
  const unsigned rows = row_mask(g, sy, sz);

  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned bytes = 0;
#pragma unroll
    for (int q = 0; q < Q; ++q)
      if (!ODD || ((rows >> row_bit(-L::ey(q), -L::ez(q))) & 1u)) bytes += row_bytes;
    mbar_expect_tx(bar, bytes);
    long long base;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      if (!ODD) {
        bulk_load(smem_addr(buf + q * P0), F + q * Np + own, row_bytes, bar);
      } else if (row_of(g, sy, sz, -L::ey(q), -L::ez(q), base)) {
        bulk_load(smem_addr(buf + q * P0), F + L::opp(q) * Np + base, row_bytes, bar);
      }
    }
  }
  // x neighbours of this thread's node (periodic wrap inside the row)
  const int x = threadIdx.x;
  const int S0 = g.S[0];
  const bool active = x < S0;
  const int xm = x > 0 ? x - 1 : S0 - 1;
  const int xp = x < S0 - 1 ? x + 1 : 0;
  const bool vxm = x > 0 || g.per[0];
  const bool vxp = x < S0 - 1 || g.per[0];

  // the node's particle-table entries, fetched while the bulk copies fly
  const long long n = own + x;
  uint8_t flag = 0;
  float4 r1 = make_float4(0.f, 0.f, 0.f, 0.f), r2 = r1;
  if (active) {
    flag = p.tab.flag[n];
    if (flag) {
      r1 = p.tab.rec32[2 * n];
      r2 = p.tab.rec32[2 * n + 1];
    }
  }
  // one thread polls the mbarrier (bounded), the others wait at the block barrier
  __shared__ int ready;
  if (threadIdx.x == 0) {
    int ok = 0;
    for (long long it = 0; it < MBAR_SPIN_LIMIT; ++it)
      if (mbar_try_wait(bar, 0)) {
        ok = 1;
        break;
      }
    if (!ok) {
      atomicOr(p.status, STATUS_TIMEOUT);
      // let the copies already issued land before the block gives up its shared memory
      for (long long it = 0; it < MBAR_SPIN_LIMIT && !mbar_try_wait(bar, 0); ++it) {
      }
    }
    ready = ok;
  }
  __syncthreads();
  if (!ready) return;

  float f[Q];
  if (active) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
      // the source node x - e_q exists: row and x neighbour
      const bool ok = ((rows >> row_bit(-cy, -cz)) & 1u) && (cx == 0 || (cx > 0 ? vxm : vxp));
      const int xs = ODD ? (cx == 0 ? x : (cx > 0 ? xm : xp)) : x;
      f[q] = ok ? Store<T>::load(buf + q * P0 + xs, sc) : 0.0f;
    }
    collide_node_lowp<L, FORCE>(f, p, n, flag, r1, r2);
  }
  __syncthreads();  // every input read before any output overwrites the rows
  if (active) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      if (!ODD) {
        Store<T>::store(buf + L::opp(q) * P0 + x, f[q], sc);
      } else {
        const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
        const bool ok = ((rows >> row_bit(cy, cz)) & 1u) && (cx == 0 || (cx > 0 ? vxp : vxm));
        const int xt = cx == 0 ? x : (cx > 0 ? xp : xm);
        if (ok) Store<T>::store(buf + q * P0 + xt, f[q], sc);
      }
    }
  }
  fence_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    long long base;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      if (!ODD) {
        bulk_store(F + q * Np + own, smem_addr(buf + q * P0), row_bytes);
      } else if (row_of(g, sy, sz, L::ey(q), L::ez(q), base)) {
        bulk_store(F + q * Np + base, smem_addr(buf + q * P0), row_bytes);
      }
    }
    bulk_commit();
    bulk_wait_all();
  }
}

template <class L, typename T>
static cudaError_t launch_lowp(const CollideParams& p, int odd, cudaStream_t st) {
  if (p.g.S[0] <= STAGED_MAX_ROW && p.g.S[2] <= 65535) {
    const unsigned threads = (unsigned)((p.g.S[0] + 31) / 32 * 32);
    const size_t smem = (size_t)L::Q * p.g.P0 * sizeof(T) + 16;
    const dim3 rows((unsigned)p.g.S[1], (unsigned)p.g.S[2]);
    if (odd) {
      if (p.has_force)
        collide_staged_kernel<L, T, true, true><<<rows, threads, smem, st>>>(p);
      else
        collide_staged_kernel<L, T, true, false><<<rows, threads, smem, st>>>(p);
    } else {
      if (p.has_force)
        collide_staged_kernel<L, T, false, true><<<rows, threads, smem, st>>>(p);
      else
        collide_staged_kernel<L, T, false, false><<<rows, threads, smem, st>>>(p);
    }
    return cudaGetLastError();
  }
  dim3 block(128);
  dim3 grid((unsigned)(((p.g.S[0] + block.x - 1) / block.x) * (long long)p.g.S[1] * p.g.S[2]));
  if (odd) {
    if (p.has_force)
      collide_lowp_kernel<L, T, true, true><<<grid, block, 0, st>>>(p);
    else
      collide_lowp_kernel<L, T, true, false><<<grid, block, 0, st>>>(p);
  } else {
    if (p.has_force)
      collide_lowp_kernel<L, T, false, true><<<grid, block, 0, st>>>(p);
    else
      collide_lowp_kernel<L, T, false, false><<<grid, block, 0, st>>>(p);
  }
  return cudaGetLastError();
}

cudaError_t launch_collide_f32(const CollideParams& p, int odd, cudaStream_t st) {
  return p.g.dim == 2 ? launch_lowp<D2Q9, float>(p, odd, st) : launch_lowp<D3Q19, float>(p, odd, st);
}
cudaError_t launch_collide_f16(const CollideParams& p, int odd, cudaStream_t st) {
  return p.g.dim == 2 ? launch_lowp<D2Q9, __half>(p, odd, st)
                      : launch_lowp<D3Q19, __half>(p, odd, st);
}

// ------------------------------------------------------------------ Zou-He
// The ZouHeBC closures on deviations g = f - w.  Each density sum of the
// reference weighs the known populations so that the w_q parts add up to
// exactly 1, hence rho = (1 + S_g)/(1 -/+ u) with S_g the same sum over g; all
// other lines are differences of populations with equal weights and carry
// over unchanged.
__device__ void zh_apply_g(int kind, float* f, float p0) {
  const float o3 = 1.0f / 3.0f, o6 = 1.0f / 6.0f, t3 = 2.0f / 3.0f;
  switch (kind) {
    case FACE_VEL2_XN: {
      const float ux = p0;
      float rho = (1.0f + (f[0] + f[2] + f[4] + 2.0f * (f[3] + f[6] + f[7]))) / (1.0f - ux);
      f[5] = f[7] + 0.5f * (f[4] - f[2]) + rho * ux * o6;
      f[8] = f[6] + 0.5f * (f[2] - f[4]) + rho * ux * o6;
      f[1] = f[3] + t3 * rho * ux;
    } break;
    case FACE_VEL2_XP: {
      const float ux = p0;
      float rho = (1.0f + (f[0] + f[2] + f[4] + 2.0f * (f[1] + f[5] + f[8]))) / (1.0f - ux);
      f[7] = f[5] + 0.5f * (f[2] - f[4]) - rho * ux * o6;
      f[6] = f[8] + 0.5f * (f[4] - f[2]) - rho * ux * o6;
      f[3] = f[1] - t3 * rho * ux;
    } break;
    case FACE_DENS2_XP: {
      const float rb = p0;
      float ux = ((1.0f - rb) + (f[0] + f[2] + f[4] + 2.0f * (f[1] + f[5] + f[8]))) / rb;
      f[6] = f[8] + 0.5f * (f[4] - f[2]) - rb * ux * o6;
      f[7] = f[5] + 0.5f * (f[2] - f[4]) - rb * ux * o6;
      f[3] = f[1] - t3 * rb * ux;
    } break;
    case FACE_VEL2_YN: {
      const float ux = p0;
      float rho = 1.0f + (f[0] + f[3] + f[1] + 2.0f * (f[8] + f[4] + f[7]));
      f[6] = f[8] + 0.5f * (f[1] - f[3]) - rho * ux * 0.5f;
      f[5] = f[7] + 0.5f * (f[3] - f[1]) + rho * ux * 0.5f;
      f[2] = f[4];
    } break;
    case FACE_VEL2_YP: {
      const float ux = p0;
      float rho = 1.0f + (f[0] + f[3] + f[1] + 2.0f * (f[6] + f[2] + f[5]));
      f[7] = f[5] + 0.5f * (f[1] - f[3]) - rho * ux * 0.5f;
      f[8] = f[6] + 0.5f * (f[3] - f[1]) + rho * ux * 0.5f;
      f[4] = f[2];
    } break;
    case FACE_VEL3_XN: {
      const float ux = p0;
      float rho = (1.0f + (f[0] + f[3] + f[4] + f[5] + f[6] + f[11] + f[17] + f[18] + f[12] +
                           2.0f * (f[2] + f[14] + f[8] + f[16] + f[10]))) / (1.0f - ux);
      float Nyx = 0.5f * (f[3] + f[11] + f[17] - (f[4] + f[18] + f[12]));
      float Nzx = 0.5f * (f[5] + f[18] + f[11] - (f[6] + f[17] + f[12]));
      f[1] = f[2] + o3 * rho * ux;
      f[13] = f[14] + rho * o6 * ux + Nyx;
      f[7] = f[8] + rho * o6 * ux - Nyx;
      f[9] = f[10] + rho * o6 * ux - Nzx;
      f[15] = f[16] + rho * o6 * ux + Nzx;
    } break;
    case FACE_VEL3_XP: {
      const float ux = p0;
      float rho = (1.0f + (f[0] + f[3] + f[4] + f[5] + f[6] + f[11] + f[17] + f[18] + f[12] +
                           2.0f * (f[1] + f[7] + f[13] + f[9] + f[15]))) / (1.0f + ux);
      float Nyx = 0.5f * (f[3] + f[11] + f[17] - (f[4] + f[18] + f[12]));
      float Nzx = 0.5f * (f[5] + f[18] + f[11] - (f[6] + f[17] + f[12]));
      f[2] = f[1] - o3 * rho * ux;
      f[14] = f[13] - rho * o6 * ux - Nyx;
      f[8] = f[7] - rho * o6 * ux + Nyx;
      f[10] = f[9] - rho * o6 * ux + Nzx;
      f[16] = f[15] - rho * o6 * ux - Nzx;
    } break;
    case FACE_DENS3_XP: {
      const float rb = p0;
      float ux = ((1.0f - rb) + (f[0] + f[3] + f[4] + f[5] + f[6] + f[11] + f[17] + f[18] + f[12] +
                                 2.0f * (f[1] + f[7] + f[13] + f[9] + f[15]))) / rb;
      float Nyx = 0.5f * (f[3] + f[11] + f[17] - (f[4] + f[18] + f[12]));
      float Nzx = 0.5f * (f[5] + f[18] + f[11] - (f[6] + f[17] + f[12]));
      f[2] = f[1] - o3 * rb * ux;
      f[14] = f[13] - rb * o6 * ux - Nyx;
      f[8] = f[7] - rb * o6 * ux + Nyx;
      f[10] = f[9] - rb * o6 * ux + Nzx;
      f[16] = f[15] - rb * o6 * ux - Nzx;
    } break;
    case FACE_VEL3_YN: {  // tangential wall velocity ux, uy = uz = 0
      const float ux = p0;
      float rho = 1.0f + (f[0] + f[1] + f[2] + f[5] + f[6] + f[9] + f[15] + f[16] + f[10] +
                          2.0f * (f[4] + f[13] + f[8] + f[18] + f[12]));
      float Nxy = 0.5f * (f[1] + f[9] + f[15] - (f[2] + f[16] + f[10])) - o3 * rho * ux;
      float Nzy = 0.5f * (f[5] + f[9] + f[16] - (f[6] + f[15] + f[10]));
      f[3] = f[4];
      f[7] = f[8] + rho * o6 * ux - Nxy;
      f[14] = f[13] - rho * o6 * ux + Nxy;
      f[11] = f[12] - Nzy;
      f[17] = f[18] + Nzy;
    } break;
    case FACE_VEL3_YP: {
      const float ux = p0;
      float rho = 1.0f + (f[0] + f[1] + f[2] + f[5] + f[6] + f[9] + f[15] + f[16] + f[10] +
                          2.0f * (f[3] + f[7] + f[14] + f[11] + f[17]));
      float Nxy = 0.5f * (f[1] + f[9] + f[15] - (f[2] + f[16] + f[10])) - o3 * rho * ux;
      float Nzy = 0.5f * (f[5] + f[9] + f[16] - (f[6] + f[15] + f[10]));
      f[4] = f[3];
      f[8] = f[7] - rho * o6 * ux + Nxy;
      f[13] = f[14] + rho * o6 * ux - Nxy;
      f[12] = f[11] + Nzy;
      f[18] = f[17] - Nzy;
    } break;
    case FACE_VEL3_ZN: {
      const float ux = p0;
      float rho = 1.0f + (f[0] + f[1] + f[2] + f[3] + f[4] + f[7] + f[13] + f[14] + f[8] +
                          2.0f * (f[6] + f[15] + f[10] + f[17] + f[12]));
      float Nxz = 0.5f * (f[1] + f[7] + f[13] - (f[2] + f[14] + f[8])) - o3 * rho * ux;
      float Nyz = 0.5f * (f[3] + f[7] + f[14] - (f[4] + f[13] + f[8]));
      f[5] = f[6];
      f[9] = f[10] + rho * o6 * ux - Nxz;
      f[16] = f[15] - rho * o6 * ux + Nxz;
      f[11] = f[12] - Nyz;
      f[18] = f[17] + Nyz;
    } break;
    case FACE_VEL3_ZP: {
      const float ux = p0;
      float rho = 1.0f + (f[0] + f[1] + f[2] + f[3] + f[4] + f[7] + f[14] + f[8] + f[13] +
                          2.0f * (f[5] + f[9] + f[16] + f[11] + f[18]));
      float Nxz = 0.5f * (f[1] + f[7] + f[13] - (f[2] + f[14] + f[8])) - o3 * rho * ux;
      float Nyz = 0.5f * (f[3] + f[7] + f[14] - (f[4] + f[13] + f[8]));
      f[6] = f[5];
      f[15] = f[16] + rho * o6 * ux - Nxz;
      f[10] = f[9] - rho * o6 * ux + Nxz;
      f[17] = f[18] - Nyz;
      f[12] = f[11] + Nyz;
    } break;
    default:
      break;
  }
}

__device__ __forceinline__ bool face_has(const Face& fc, int sx, int sy, int sz) {
  return sx >= fc.lo[0] && sx <= fc.hi[0] && sy >= fc.lo[1] && sy <= fc.hi[1] &&
         sz >= fc.lo[2] && sz <= fc.hi[2];
}

template <class L, typename T>
__global__ void bc_lowp_kernel(BCParams p) {
  constexpr int Q = L::Q;
  const int fi = blockIdx.y;
  const Face& fc = p.face[fi];
  const int na = fc.hi[0] - fc.lo[0] + 1, nb_ = fc.hi[1] - fc.lo[1] + 1,
            nc = fc.hi[2] - fc.lo[2] + 1;
  const long long total = (long long)na * nb_ * nc;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int sx = fc.lo[0] + (int)(t % na);
  const int sy = fc.lo[1] + (int)((t / na) % nb_);
  const int sz = fc.lo[2] + (int)(t / ((long long)na * nb_));
  for (int k = 0; k < fi; ++k)
    if (face_has(p.face[k], sx, sy, sz)) return;
  const Geom& g = p.g;
  const Nbr nb = make_nbr(g, sx, sy, sz);
  const long long n = node_index(g, sx, sy, sz);
  T* F = static_cast<T*>(p.f);
  float f[Q];
  long long loc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    if (!nbr_ok(nb, -cx, -cy, -cz)) {
      loc[q] = -1;
    } else if (p.after_odd) {
      loc[q] = (long long)q * g.Np + n;
    } else {
      loc[q] = (long long)L::opp(q) * g.Np + n + nbr_off(nb, -cx, -cy, -cz);
    }
    f[q] = loc[q] >= 0 ? Store<T>::load(F + loc[q], p.scale16) : 0.0f;
  }
  for (int k = fi; k < p.nfaces; ++k)
    if (face_has(p.face[k], sx, sy, sz)) zh_apply_g(p.face[k].kind, f, (float)p.face[k].p0);
#pragma unroll
  for (int q = 0; q < Q; ++q)
    if (loc[q] >= 0) Store<T>::store(F + loc[q], f[q], p.scale16);
}

template <typename T>
static cudaError_t launch_bc_lowp(const BCParams& p, cudaStream_t st) {
  if (p.nfaces == 0) return cudaSuccess;
  long long maxn = 0;
  for (int k = 0; k < p.nfaces; ++k) {
    const Face& fc = p.face[k];
    long long c = (long long)(fc.hi[0] - fc.lo[0] + 1) * (fc.hi[1] - fc.lo[1] + 1) *
                  (fc.hi[2] - fc.lo[2] + 1);
    if (c > maxn) maxn = c;
  }
  if (maxn <= 0) return cudaSuccess;
  dim3 block(128);
  dim3 grid((unsigned)((maxn + 127) / 128), (unsigned)p.nfaces);
  if (p.g.dim == 2)
    bc_lowp_kernel<D2Q9, T><<<grid, block, 0, st>>>(p);
  else
    bc_lowp_kernel<D3Q19, T><<<grid, block, 0, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_bc_f32(const BCParams& p, cudaStream_t st) { return launch_bc_lowp<float>(p, st); }
cudaError_t launch_bc_f16(const BCParams& p, cudaStream_t st) { return launch_bc_lowp<__half>(p, st); }

}  // namespace lbmpsm
