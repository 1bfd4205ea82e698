// collide_lowp.cu -- FP32-collision paths of the fused collide / A-A stream
// kernel and the Zou-He face kernel.
//
// Populations are stored as deviations g_q = f_q - w_q*rho0 (rho0 = 1): in
// FP32 (LBMPSM_STORAGE_FP32), in FP16 scaled by scale16
// (LBMPSM_STORAGE_FP16), or in BF16 (LBMPSM_STORAGE_BF16: FP32's exponent
// range, so no scale, and 8 significant bits against FP16's 11).  The collision runs in FP32 on the deviations, which
// keeps the small differences f - feq of a low-Mach flow well resolved; the
// algebra is the reference's (src/LBM_PSM_BGK_dynamics.h:40-114,
// src/LBM_PSM_dynamics.h:43-116) with the w_q*rho0 parts cancelled:
//   feq_q - w_q = w_q (drho + rho (3 e.u + 4.5 (e.u)^2 - 1.5 u.u)).
// Node forces of PSM nodes are written in FP32 and reduced per particle in
// FP64 (particles.cu).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdlib>

#include "lbmpsm_internal.cuh"

namespace lbmpsm {

// load / store: deviations in FP32.  raw_load / raw_store: the stored value
// times 2^-SH unscaled, i.e. the deviation times 2^SH, which the collide
// kernels take as is (collide_node_lowp's SH).
template <typename T>
struct Store;
template <>
struct Store<float> {
  static constexpr int SH = 0;
  __device__ __forceinline__ static float load(const float* p, float) { return *p; }
  __device__ __forceinline__ static void store(float* p, float v, float) { *p = v; }
  __device__ __forceinline__ static float raw_load(const float* p) { return *p; }
  __device__ __forceinline__ static void raw_store(float* p, float v) { *p = v; }
};
template <>
struct Store<__nv_bfloat16> {
  static constexpr int SH = 0;
  __device__ __forceinline__ static float load(const __nv_bfloat16* p, float) {
    return __bfloat162float(*p);
  }
  __device__ __forceinline__ static void store(__nv_bfloat16* p, float v, float) {
    *p = __float2bfloat16_rn(v);
  }
  __device__ __forceinline__ static float raw_load(const __nv_bfloat16* p) {
    return __bfloat162float(*p);
  }
  __device__ __forceinline__ static void raw_store(__nv_bfloat16* p, float v) {
    *p = __float2bfloat16_rn(v);
  }
};
template <>
struct Store<__half> {
  static constexpr int SH = FP16_SCALE_LOG2;
  __device__ __forceinline__ static float load(const __half* p, float scale) {
    return __half2float(*p) * (1.0f / scale);
  }
  __device__ __forceinline__ static void store(__half* p, float v, float scale) {
    *p = __float2half_rn(v * scale);
  }
  __device__ __forceinline__ static float raw_load(const __half* p) { return __half2float(*p); }
  __device__ __forceinline__ static void raw_store(__half* p, float v) {
    *p = __float2half_rn(v);
  }
};

// e_q . v for compile-time components (folded once the q loop is unrolled;
// -0 is the identity of IEEE addition, so the leading term costs nothing)
__device__ __forceinline__ float sgn_add(float s, int c, float v) {
  return c == 0 ? s : (c > 0 ? s + v : s - v);
}
__device__ __forceinline__ float edot(int cx, int cy, int cz, float vx, float vy, float vz) {
  return sgn_add(sgn_add(sgn_add(-0.0f, cx, vx), cy, vy), cz, vz);
}

// Collision of one node on its Q deviations f[], in place
// (src/LBM_PSM_BGK_dynamics.h:40-114, src/LBM_PSM_dynamics.h:43-116).
//
// With Omega_s^n = feq(rho, u_s^n) - f + (1 - omega)(f - feq) and
// sum_n B_n = B_t the reference update
//   f' = f + (1 - B_t) omega (feq - f) + sum_n B_n Omega_s^n + F_q
// equals, term for term in exact arithmetic,
//   f' = f + omega (feq - f) + F_q + sum_n B_n (feq(rho, u_s^n) - feq(rho, u)),
// and the difference of the two equilibria of direction q is
//   w_q rho [a (3 + 4.5 b) - 1.5 (|u_s|^2 - |u|^2)],  a = e.(u_s - u), b = e.(u_s + u),
// which is how it is evaluated here (no cancellation between two O(w)
// equilibria).  The node force of slot n, -B_n sum_q Omega_s^n e_q, is by the
// moments of the D2Q9/D3Q19 equilibria (sum_q feq(rho, v) e_q = rho v)
//   -B_n [rho u_s^n - j + omega F/2]       (j including the F/2 shift),
// so it needs no per-direction accumulation.
//
// The warp takes the plain BGK loop when none of its nodes is a PSM node,
// the one-slot loop when none holds two particles, else the two-slot loop;
// an unused slot has B = 0 and leaves f' bit-identical to the shorter loop.
//
// SH > 0: f[] holds the deviations times S = 2^SH (FP16 storage's scale) and
// is left scaled the same way.  Every quantity is then either the unscaled
// one or exactly S times it (drho and j are summed scaled, the equilibrium
// weights carry S); a power-of-two factor commutes with IEEE rounding, so
// the results are bit for bit those of scaling on every load and store.
template <class L, bool FORCE, bool MACRO = true, int SH = 0>
__device__ __forceinline__ void collide_node_lowp(float (&f)[L::Q], const CollideParams& p,
                                                  const BoxParams& bp, long long n, uint8_t flag,
                                                  float4 r1, float4 r2) {
  constexpr int Q = L::Q;
  constexpr float S = (float)(1 << SH), Si = 1.0f / (float)(1 << SH);
  float dS = -0.0f, jx = -0.0f, jy = -0.0f, jz = -0.0f;  // scaled by S
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    dS += f[q];
    jx = sgn_add(jx, L::ex(q), f[q]);
    jy = sgn_add(jy, L::ey(q), f[q]);
    jz = sgn_add(jz, L::ez(q), f[q]);
  }
  // the unscaling products are exact; __fmul_rn keeps them out of FMA
  // contraction, which would round the neighbouring terms differently
  const float drho = SH ? __fmul_rn(dS, Si) : dS;
  const float Fx = bp.F_f[0], Fy = bp.F_f[1], Fz = bp.F_f[2];
  if (FORCE) {
    jx += (0.5f * S) * Fx;
    jy += (0.5f * S) * Fy;
    jz += (0.5f * S) * Fz;
  }
  const float rho = 1.0f + drho;
  const float inv = SH ? __fmul_rn(__frcp_rn(rho), Si) : __frcp_rn(rho);
  const float ux = jx * inv, uy = jy * inv, uz = jz * inv;
  if (MACRO && p.store_macro) {
    p.rho_out[n] = 1.0 + (double)drho;
    p.u_out[3 * n + 0] = ux;
    p.u_out[3 * n + 1] = uy;
    p.u_out[3 * n + 2] = uz;
  }
  const float usq15 = 1.5f * (ux * ux + uy * uy + uz * uz);
  const float omega = bp.omega_f;
  const float gpref = bp.gpref_f;
  const float uF = FORCE ? ux * Fx + uy * Fy + uz * Fz : 0.0f;
  const float dr_u = drho - rho * usq15;

  // BGK part of direction q: f + omega (feq - f) + F_q
#define LBMPSM_BGK_Q(q)                                                              \
  const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);                            \
  const float w = (float)L::w(q) * S;                                               \
  const float eu = edot(cx, cy, cz, ux, uy, uz);                                    \
  const float geq = w * fmaf(rho * eu, fmaf(4.5f, eu, 3.0f), dr_u);                 \
  float bgk = fmaf(omega, geq - f[q], f[q]);                                        \
  if (FORCE) {                                                                      \
    const float eF = edot(cx, cy, cz, Fx, Fy, Fz);                                  \
    bgk += gpref * w * fmaf(9.0f * eu, eF, 3.0f * (eF - uF));                       \
  }

  const unsigned act = __activemask();
  const bool psm = flag != 0;
  if (!__any_sync(act, psm)) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      LBMPSM_BGK_Q(q)
      f[q] = bgk;
    }
    return;
  }
  const bool has1 = (flag & 1) != 0, has2 = (flag & 2) != 0;
  float B1 = has1 ? r1.x : 0.0f;
  float B2 = has2 ? r2.x : 0.0f;
  if (p.weighting == 1) {  // Noble-Torczynski weighting (opt-in)
    const float tm = bp.tm_f;
    if (has1) B1 = B1 * tm / ((1.0f - B1) + tm);
    if (has2) B2 = B2 * tm / ((1.0f - B2) + tm);
  }
  const float Bt = B1 + B2;
  if (Bt > 1.0f) {
    B1 = B1 / Bt;
    B2 = B2 / Bt;
  }
  const float s1x = has1 ? r1.y : 0.0f, s1y = has1 ? r1.z : 0.0f, s1z = has1 ? r1.w : 0.0f;
  const float s2x = has2 ? r2.y : 0.0f, s2y = has2 ? r2.z : 0.0f, s2z = has2 ? r2.w : 0.0f;
  const float B1r = B1 * rho, B2r = B2 * rho;
  const float dq1 = fmaf(1.5f, s1x * s1x + s1y * s1y + s1z * s1z, -usq15);
  const float dq2 = fmaf(1.5f, s2x * s2x + s2y * s2y + s2z * s2z, -usq15);
  if (!__any_sync(act, has2)) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      LBMPSM_BGK_Q(q)
      const float a1 = edot(cx, cy, cz, s1x - ux, s1y - uy, s1z - uz);
      const float b1 = edot(cx, cy, cz, s1x + ux, s1y + uy, s1z + uz);
      f[q] = fmaf(B1r * w, fmaf(a1, fmaf(4.5f, b1, 3.0f), -dq1), bgk);
    }
  } else {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      LBMPSM_BGK_Q(q)
      const float a1 = edot(cx, cy, cz, s1x - ux, s1y - uy, s1z - uz);
      const float b1 = edot(cx, cy, cz, s1x + ux, s1y + uy, s1z + uz);
      const float a2 = edot(cx, cy, cz, s2x - ux, s2y - uy, s2z - uz);
      const float b2 = edot(cx, cy, cz, s2x + ux, s2y + uy, s2z + uz);
      bgk = fmaf(B1r * w, fmaf(a1, fmaf(4.5f, b1, 3.0f), -dq1), bgk);
      f[q] = fmaf(B2r * w, fmaf(a2, fmaf(4.5f, b2, 3.0f), -dq2), bgk);
    }
  }
#undef LBMPSM_BGK_Q
  if (psm) {
    if (SH) {  // the node force needs j itself
      jx = __fmul_rn(jx, Si);
      jy = __fmul_rn(jy, Si);
      jz = __fmul_rn(jz, Si);
    }
    const float hx = 0.5f * omega * Fx, hy = 0.5f * omega * Fy, hz = 0.5f * omega * Fz;
    float* nf = static_cast<float*>(p.tab.nodeF) + 6 * n;
    nf[0] = -B1 * (fmaf(rho, s1x, -jx) + (FORCE ? hx : 0.0f));
    nf[1] = -B1 * (fmaf(rho, s1y, -jy) + (FORCE ? hy : 0.0f));
    nf[2] = -B1 * (fmaf(rho, s1z, -jz) + (FORCE ? hz : 0.0f));
    nf[3] = -B2 * (fmaf(rho, s2x, -jx) + (FORCE ? hx : 0.0f));
    nf[4] = -B2 * (fmaf(rho, s2y, -jy) + (FORCE ? hy : 0.0f));
    nf[5] = -B2 * (fmaf(rho, s2z, -jz) + (FORCE ? hz : 0.0f));
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
  float f[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    const bool ok = nbr_ok(nb, -cx, -cy, -cz);
    if (!ODD) {
      f[q] = ok ? Store<T>::raw_load(F + q * Np + n) : 0.0f;
    } else {
      const int o = nbr_off(nb, -cx, -cy, -cz);
      f[q] = ok ? Store<T>::raw_load(F + L::opp(q) * Np + n + o) : 0.0f;
    }
  }
  const uint8_t flag = p.tab.flag[n];
  float4 r1 = make_float4(0.f, 0.f, 0.f, 0.f), r2 = r1;
  if (flag) {
    r1 = p.tab.rec32[2 * n];
    r2 = p.tab.rec32[2 * n + 1];
  }
  collide_node_lowp<L, FORCE, true, Store<T>::SH>(f, p, p.box[box_of_z(g, sz)], n, flag, r1, r2);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    if (!ODD) {
      Store<T>::raw_store(F + L::opp(q) * Np + n, f[q]);
    } else {
      if (nbr_ok(nb, cx, cy, cz)) Store<T>::raw_store(F + q * Np + n + nbr_off(nb, cx, cy, cz), f[q]);
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
// every bulk store group of this thread has finished reading shared memory
__device__ __forceinline__ void bulk_wait_read0() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

constexpr int STAGED_MAX_ROW = 256;      // nodes per x-row handled by one staged block
constexpr long long MBAR_SPIN_LIMIT = 1ll << 26;

// neighbour row (dy, dz) of row (sy, sz); false when it does not exist
// (z wraps or ends within the row's box of a batched ensemble)
__device__ __forceinline__ bool row_of(const Geom& g, int sy, int sz, int dy, int dz,
                                       long long& base) {
  const int z0 = box_of_z(g, sz) * g.bz;
  int y = sy + dy, z = sz - z0 + dz;
  if (y < 0 || y >= g.S[1]) {
    if (!g.per[1]) return false;
    y = y < 0 ? y + g.S[1] : y - g.S[1];
  }
  if (z < 0 || z >= g.bz) {
    if (!g.per[2]) return false;
    z = z < 0 ? z + g.bz : z - g.bz;
  }
  base = ((long long)(z0 + z) * g.S[1] + y) * g.P0;
  return true;
}

// bit (dy+1)*3 + (dz+1) set when row (sy+dy, sz+dz) exists
__device__ __forceinline__ unsigned row_mask(const Geom& g, int sy, int sz) {
  unsigned m = 0;
  const int lz = sz - box_of_z(g, sz) * g.bz;  // plane within the box
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz) {
      const int y = sy + dy, z = lz + dz;
      const bool oky = (y >= 0 && y < g.S[1]) || g.per[1];
      const bool okz = (z >= 0 && z < g.bz) || g.per[2];
      if (oky && okz) m |= 1u << ((dy + 1) * 3 + (dz + 1));
    }
  return m;
}
__host__ __device__ constexpr int row_bit(int dy, int dz) { return (dy + 1) * 3 + (dz + 1); }

// next row of a block's sequence: rows r, r + G, r + 2G, ... with
// G = dz * S1 + dy, kept as (sy, sz) without division
__device__ __forceinline__ void next_row(int& sy, int& sz, int dy, int dz, int S1) {
  sy += dy;
  sz += dz;
  if (sy >= S1) {
    sy -= S1;
    sz += 1;
  }
}

__device__ __forceinline__ void mbar_arrive(unsigned bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// barrier over nthreads threads that also ANDs a predicate across them
__device__ __forceinline__ bool named_bar_and(int id, int nthreads, bool v) {
  int r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, %2, %3, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((int)v), "r"(id), "r"(nthreads)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned phase,
                                                  long long limit = MBAR_SPIN_LIMIT) {
  for (long long it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}
// The same wait, also ended when *abort (a shared-memory flag) is set.
__device__ __forceinline__ bool mbar_wait_abortable(unsigned bar, unsigned phase,
                                                    const volatile int* abort) {
  for (long long it = 0; it < MBAR_SPIN_LIMIT; ++it) {
    if (mbar_try_wait(bar, phase)) return true;
    if (*abort) return false;
  }
  return false;
}

// Warp-specialised row pipeline of the collide / A-A stream step.  A
// persistent grid; every block walks its x-rows r, r + G, r + 2G, ... through
// NST shared-memory stages of Q population rows each.
//   producer warp (the last warp): lane q moves direction q -- it stores the
//     outputs of row k - NST from stage s once the consumers are done with
//     it, waits until that store has read the stage, then loads the inputs of
//     row k into it; so the loads run up to NST - 1 rows ahead.
//   consumer warps: one thread per node of the row; wait for the stage,
//     collide, write the outputs back into the stage in place, signal done.
//   even step: own row, slot q in, slot opp(q) out;
//   odd step : row -e_q, slot opp(q) in -> row +e_q, slot q out.
// Within a row the x-shifts of streaming are shared-memory index offsets.
// The A-A pattern makes each block the only reader and writer of the
// locations it moves, so blocks never wait for one another.  Every wait is
// bounded: on expiry the block records STATUS_TIMEOUT, lets the copies it
// issued land (bounded too) and returns.  Consumers that give up on a stage
// (after p.full_wait_limit polls) raise a shared abort flag, which ends the
// producer's wait for their signal at once; the producer then waits, with
// its own long limit, only for the loads it has issued.
template <class L, typename T, bool ODD, bool FORCE, int NST, int MINB>
__global__ void __launch_bounds__(STAGED_MAX_ROW + 32, MINB) collide_pipe_kernel(CollideParams p) {
  static_assert(NST >= 2, "stages");
  constexpr int Q = L::Q;
  static_assert(Q <= 32, "one producer lane per direction");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long full[NST], done[NST];
  __shared__ int s_abort;  // set by the consumers when they give up
  const Geom& g = p.g;
  const int P0 = g.P0, S0 = g.S[0], S1 = g.S[1];
  const int R = S1 * g.S[2];
  const int G = gridDim.x;
  const int gdy = p.pipe.dy, gdz = p.pipe.dz;
  const int ncons = (int)blockDim.x - 32;
  const unsigned row_bytes = (unsigned)(P0 * sizeof(T));
  const unsigned stage_bytes = (unsigned)Q * row_bytes;
  const unsigned smem0 = smem_addr(smem_raw);
  T* __restrict__ F = static_cast<T*>(p.f);
  const int tid = threadIdx.x;

  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < NST; ++s) {
      mbar_init(smem_addr(&full[s]), 1);
      mbar_init(smem_addr(&done[s]), (unsigned)ncons);
    }
    s_abort = 0;
    fence_mbar_init();
  }
  __syncthreads();

  if (tid >= ncons) {
    // ------------------------------------------------------------ producer
    const int lane = tid - ncons;
    const bool mine = lane < Q;
    int ey = 0, ez = 0, qo = 0;
#pragma unroll
    for (int qq = 0; qq < Q; ++qq)
      if (qq == lane) {
        ey = L::ey(qq);
        ez = L::ez(qq);
        qo = L::opp(qq);
      }
    const long long Np = g.Np;
    int ly = blockIdx.x % S1, lz = blockIdx.x / S1;  // next row to load
    int sy = ly, sz = lz;                            // next row to store
    int ls = 0, lph = 0;                             // its stage and parity
    int ss = 0, sph = 0;
    int loaded = 0, stored = 0;
    bool ok = true;
    const int K = blockIdx.x < (unsigned)R ? (R - 1 - (int)blockIdx.x) / G + 1 : 0;
    while (stored < K) {
      const bool can_load = loaded < K && loaded - stored < NST;
      if (!can_load) {
        // store the oldest row once the consumers are done with it
        // one decision for the whole warp (its lanes poll independently)
        ok = __all_sync(0xffffffffu, mbar_wait_abortable(smem_addr(&done[ss]), sph, &s_abort));
        if (!ok) break;
        long long base = 0;
        // back where it was loaded from (the odd step's outputs were written
        // into the rows their locations came from)
        const bool ex = mine && (ODD ? row_of(g, sy, sz, -ey, -ez, base)
                                     : (base = ((long long)sz * S1 + sy) * P0, true));
        if (ex)
          bulk_store(F + (ODD ? qo : lane) * Np + base, smem0 + ss * stage_bytes + lane * row_bytes,
                     row_bytes);
        bulk_commit();
        next_row(sy, sz, gdy, gdz, S1);
        ++stored;
        if (++ss == NST) {
          ss = 0;
          sph ^= 1;
        }
        continue;
      }
      if (loaded >= NST) {
        // stage ls held row loaded - NST, stored just before: wait until the
        // store has read it (each lane its own bulk group)
        bulk_wait_read0();
        __syncwarp();
      }
      long long base = 0;
      const bool ex = mine && (ODD ? row_of(g, ly, lz, -ey, -ez, base)
                                   : (base = ((long long)lz * S1 + ly) * P0, true));
      const unsigned cnt = __popc(__ballot_sync(0xffffffffu, ex));
      const unsigned bar = smem_addr(&full[ls]);
      if (lane == 0) mbar_expect_tx(bar, cnt * row_bytes);
      __syncwarp();
      if (ex)
        bulk_load(smem0 + ls * stage_bytes + lane * row_bytes, F + (ODD ? qo : lane) * Np + base,
                  row_bytes, bar);
      next_row(ly, lz, gdy, gdz, S1);
      ++loaded;
      if (++ls == NST) {
        ls = 0;
        lph ^= 1;
      }
    }
    if (!ok) {
      if (lane == 0) atomicOr(p.status, STATUS_TIMEOUT);
      // let the loads still in flight land: rows stored .. loaded-1
      int ts = ss, tph = sph;
      for (int k = stored; k < loaded; ++k) {
        mbar_wait_bounded(smem_addr(&full[ts]), tph);
        if (++ts == NST) {
          ts = 0;
          tph ^= 1;
        }
      }
    }
    bulk_wait_all();
    (void)lph;
    return;
  }

  // -------------------------------------------------------------- consumers
  const int x = tid;
  const bool active = x < S0;
  const int xm = x > 0 ? x - 1 : S0 - 1;
  const int xp = x < S0 - 1 ? x + 1 : 0;
  const bool vxm = x > 0 || g.per[0];
  const bool vxp = x < S0 - 1 || g.per[0];
  int cy = blockIdx.x % S1, cz = blockIdx.x / S1;
  int s = 0, ph = 0;
  for (int r = blockIdx.x; r < R; r += G) {
    const long long own = ((long long)cz * S1 + cy) * P0;
    const unsigned rows = row_mask(g, cy, cz);
    constexpr unsigned need = L::Q == 9 ? 0x92u : 0x1FFu;  // (dy, dz) rows the set uses
    const bool all_ok = (rows & need) == need && g.per[0];  // every source node exists
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
    bool ok = true;
    if (tid == 0)
      ok = mbar_wait_bounded(smem_addr(&full[s]), ph,
                             p.full_wait_limit > 0 ? p.full_wait_limit
                                                   : (p.full_wait_limit < 0 ? 0 : MBAR_SPIN_LIMIT));
    if (!named_bar_and(1, ncons, ok)) {
      if (tid == 0) {
        atomicOr(p.status, STATUS_TIMEOUT);
        *static_cast<volatile int*>(&s_abort) = 1;
        __threadfence_block();
      }
      return;
    }
    T* buf = reinterpret_cast<T*>(smem_raw + (size_t)s * stage_bytes);
    float f[Q];
    if (active) {
      if (all_ok) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int ex = L::ex(q);
          const int xs = ODD ? (ex == 0 ? x : (ex > 0 ? xm : xp)) : x;
          f[q] = Store<T>::raw_load(buf + q * P0 + xs);
        }
      } else {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int ex = L::ex(q), ey = L::ey(q), ez = L::ez(q);
          // the source node x - e_q exists: row and x neighbour
          const bool okq =
              ((rows >> row_bit(-ey, -ez)) & 1u) && (ex == 0 || (ex > 0 ? vxm : vxp));
          const int xs = ODD ? (ex == 0 ? x : (ex > 0 ? xm : xp)) : x;
          f[q] = okq ? Store<T>::raw_load(buf + q * P0 + xs) : 0.0f;
        }
      }
      collide_node_lowp<L, FORCE, true, Store<T>::SH>(f, p, p.box[box_of_z(g, cz)], n, flag, r1, r2);
    }
    // Each thread writes only the shared-memory slots it read: the even step
    // its own column; the odd step puts outgoing f_q at location (x + e_q, q),
    // which the stage holds in row opp(q) (loaded from slot q of row y + e_q)
    // at x + ex_q -- the slot this thread read as its incoming f_opp(q).  So
    // no consumer barrier separates the reads from the writes.
    if (active) {
      if (!ODD) {
#pragma unroll
        for (int q = 0; q < Q; ++q) Store<T>::raw_store(buf + L::opp(q) * P0 + x, f[q]);
      } else if (all_ok) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int ex = L::ex(q);
          const int xt = ex == 0 ? x : (ex > 0 ? xp : xm);
          Store<T>::raw_store(buf + L::opp(q) * P0 + xt, f[q]);
        }
      } else {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int ex = L::ex(q), ey = L::ey(q), ez = L::ez(q);
          const bool okq = ((rows >> row_bit(ey, ez)) & 1u) && (ex == 0 || (ex > 0 ? vxp : vxm));
          const int xt = ex == 0 ? x : (ex > 0 ? xp : xm);
          if (okq) Store<T>::raw_store(buf + L::opp(q) * P0 + xt, f[q]);
        }
      }
    }
    fence_async_smem();
    mbar_arrive(smem_addr(&done[s]));
    next_row(cy, cz, gdy, gdz, S1);
    if (++s == NST) {
      s = 0;
      ph ^= 1;
    }
  }
}

// The kernel's dynamic shared-memory limit is a property of the kernel, not
// of a launch: lattices of different row lengths share it, so it is only ever
// raised (a lattice set up later with shorter rows must not lower the limit
// that an earlier one launches with).
static cudaError_t raise_smem_limit(const void* fn, size_t smem) {
  cudaFuncAttributes a{};
  cudaError_t e = cudaFuncGetAttributes(&a, fn);
  if (e != cudaSuccess) return e;
  if ((size_t)a.maxDynamicSharedSizeBytes >= smem) return cudaSuccess;
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// ------------------------------------------------------ several lattices
// The row pipeline above over the members of a group in one persistent
// launch.  The work is a list of tiles: member m owns tiles
// [first[m], first[m+1]); a tile is k consecutive x-rows of one storage
// plane of the member (rows y0 .. y0+k-1, fewer at the plane's end), k chosen
// per member so that k rows fill the consumers (boxes of edge 32 take three
// rows per tile, 48 two, 64-96 one).  Block b takes tiles b, b + G, ...; the
// producer lane q moves direction q of each of the tile's rows with one bulk
// copy per row, the consumers take one node each (thread t: row t / S0,
// x = t % S0) and run the members' own node collision, so the results are
// those of the members' own launches.  Every member is periodic on every axis
// (rows and their neighbour rows always exist), and either every member has a
// body force or none has.  The waits are bounded as in the single-lattice
// kernel.
struct TileRef {
  int m, z, y0, k;
};
__device__ __forceinline__ TileRef tile_of(const MultiCollide& mc, const MultiMember* mem, int t) {
  int m = 0;
  while (m + 1 < mc.nm && t >= mc.first[m + 1]) ++m;
  const MultiMember& mm = mem[m];
  const unsigned lt = (unsigned)(t - mc.first[m]);
  const int z = (int)fast_div(lt, mm.ftpp);
  TileRef r;
  r.m = m;
  r.z = z;
  r.y0 = ((int)lt - z * mm.tpp) * mm.k;
  const int rest = mm.p.g.S[1] - r.y0;
  r.k = rest < mm.k ? rest : mm.k;
  return r;
}

// the widest row (nodes) a fused launch takes; 128-thread blocks at eight per
// multiprocessor (fewer registers, a few spilled to local memory, measured
// faster than four to six blocks with none)
constexpr int MULTI_MAX_ROW = 96;

template <class L, typename T, bool ODD, bool FORCE, int NST>
__global__ void __launch_bounds__(MULTI_MAX_ROW + 32, 8) collide_multi_kernel(MultiCollide mc) {
  static_assert(NST >= 2, "stages");
  constexpr int Q = L::Q;
  static_assert(Q <= 32, "one producer lane per direction");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long full[NST], done[NST];
  __shared__ int s_abort;
  // the member table in shared memory: every tile reads its member's
  // parameters, which would otherwise be a chain of global loads per tile
  __shared__ __align__(16) MultiMember s_mem[MULTI_MAX];
  const int G = gridDim.x;
  const int ncons = (int)blockDim.x - 32;
  const int tcp = mc.tcp;
  {
    const int words = mc.nm * (int)(sizeof(MultiMember) / sizeof(int));
    const int* src = reinterpret_cast<const int*>(mc.m);
    int* dst = reinterpret_cast<int*>(s_mem);
    for (int w = threadIdx.x; w < words; w += blockDim.x) dst[w] = __ldg(src + w);
  }
  const unsigned stage_bytes = (unsigned)(Q * tcp * (int)sizeof(T));
  const unsigned smem0 = smem_addr(smem_raw);
  const int tid = threadIdx.x;
  const int ntiles = mc.first[mc.nm];
  const int K = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / G + 1 : 0;

  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < NST; ++s) {
      mbar_init(smem_addr(&full[s]), 1);
      mbar_init(smem_addr(&done[s]), (unsigned)ncons);
    }
    s_abort = 0;
    fence_mbar_init();
  }
  __syncthreads();

  if (tid >= ncons) {
    // ------------------------------------------------------------ producer
    const int lane = tid - ncons;
    const bool mine = lane < Q;
    int ey = 0, ez = 0, qo = 0;
#pragma unroll
    for (int qq = 0; qq < Q; ++qq)
      if (qq == lane) {
        ey = L::ey(qq);
        ez = L::ez(qq);
        qo = L::opp(qq);
      }
    int ls = 0, ss = 0, sph = 0;
    int loaded = 0, stored = 0;
    bool ok = true;
    while (stored < K) {
      const bool can_load = loaded < K && loaded - stored < NST;
      if (!can_load) {
        // store the oldest tile once the consumers are done with it
        ok = __all_sync(0xffffffffu, mbar_wait_abortable(smem_addr(&done[ss]), sph, &s_abort));
        if (!ok) break;
        const TileRef tr = tile_of(mc, s_mem, (int)blockIdx.x + stored * G);
        if (mine) {
          const CollideParams& p = s_mem[tr.m].p;
          const Geom& g = p.g;
          T* F = static_cast<T*>(p.f);
          const unsigned row_bytes = (unsigned)(g.P0 * (int)sizeof(T));
          for (int r = 0; r < tr.k; ++r) {
            long long base = ((long long)tr.z * g.S[1] + tr.y0 + r) * g.P0;
            if (ODD) row_of(g, tr.y0 + r, tr.z, -ey, -ez, base);  // where it was loaded from
            bulk_store(F + (ODD ? qo : lane) * g.Np + base,
                       smem0 + ss * stage_bytes + (unsigned)((lane * tcp + r * g.P0) * (int)sizeof(T)),
                       row_bytes);
          }
        }
        bulk_commit();
        ++stored;
        if (++ss == NST) {
          ss = 0;
          sph ^= 1;
        }
        continue;
      }
      if (loaded >= NST) {
        // the stage held the tile stored just before: wait until the store
        // has read it (each lane its own bulk group)
        bulk_wait_read0();
        __syncwarp();
      }
      const TileRef tr = tile_of(mc, s_mem, (int)blockIdx.x + loaded * G);
      const CollideParams& p = s_mem[tr.m].p;
      const Geom& g = p.g;
      const unsigned row_bytes = (unsigned)(g.P0 * (int)sizeof(T));
      const unsigned bar = smem_addr(&full[ls]);
      if (lane == 0) mbar_expect_tx(bar, (unsigned)(Q * tr.k) * row_bytes);
      __syncwarp();
      if (mine) {
        const T* F = static_cast<const T*>(p.f);
        for (int r = 0; r < tr.k; ++r) {
          long long base = ((long long)tr.z * g.S[1] + tr.y0 + r) * g.P0;
          if (ODD) row_of(g, tr.y0 + r, tr.z, -ey, -ez, base);
          bulk_load(smem0 + ls * stage_bytes + (unsigned)((lane * tcp + r * g.P0) * (int)sizeof(T)),
                    F + (ODD ? qo : lane) * g.Np + base, row_bytes, bar);
        }
      }
      ++loaded;
      if (++ls == NST) ls = 0;
    }
    if (!ok) {
      if (lane == 0) atomicOr(mc.status, STATUS_TIMEOUT);
      // let the loads still in flight land: tiles stored .. loaded-1
      int ts = ss, tph = sph;
      for (int k = stored; k < loaded; ++k) {
        mbar_wait_bounded(smem_addr(&full[ts]), tph);
        if (++ts == NST) {
          ts = 0;
          tph ^= 1;
        }
      }
    }
    bulk_wait_all();
    return;
  }

  // -------------------------------------------------------------- consumers
  int s = 0, ph = 0;
  for (int j = 0; j < K; ++j) {
    const TileRef tr = tile_of(mc, s_mem, (int)blockIdx.x + j * G);
    const CollideParams& p = s_mem[tr.m].p;
    const Geom& g = p.g;
    const int S0 = g.S[0], P0 = g.P0;
    const int r = tid / S0;
    const int x = tid - r * S0;
    const bool active = r < tr.k;
    const int xm = x > 0 ? x - 1 : S0 - 1;
    const int xp = x < S0 - 1 ? x + 1 : 0;
    const long long n = ((long long)tr.z * g.S[1] + tr.y0 + r) * P0 + x;
    uint8_t flag = 0;
    float4 r1 = make_float4(0.f, 0.f, 0.f, 0.f), r2 = r1;
    if (active) {
      flag = p.tab.flag[n];
      if (flag) {
        r1 = p.tab.rec32[2 * n];
        r2 = p.tab.rec32[2 * n + 1];
      }
    }
    bool ok = true;
    if (tid == 0)
      ok = mbar_wait_bounded(smem_addr(&full[s]), ph,
                             mc.full_wait_limit > 0 ? mc.full_wait_limit
                                                    : (mc.full_wait_limit < 0 ? 0 : MBAR_SPIN_LIMIT));
    if (!named_bar_and(1, ncons, ok)) {
      if (tid == 0) {
        atomicOr(mc.status, STATUS_TIMEOUT);
        *static_cast<volatile int*>(&s_abort) = 1;
        __threadfence_block();
      }
      return;
    }
    T* buf = reinterpret_cast<T*>(smem_raw + (size_t)s * stage_bytes) + r * P0;
    float f[Q];
    if (active) {
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int ex = L::ex(q);
        const int xs = ODD ? (ex == 0 ? x : (ex > 0 ? xm : xp)) : x;
        f[q] = Store<T>::raw_load(buf + q * tcp + xs);
      }
      // every member has a body force, or none has (the host checks)
      collide_node_lowp<L, FORCE, false, Store<T>::SH>(f, p, p.box[box_of_z(g, tr.z)], n, flag, r1, r2);
    }
    // each thread writes only the slots it read (collide_pipe_kernel)
    if (active) {
      if (!ODD) {
#pragma unroll
        for (int q = 0; q < Q; ++q) Store<T>::raw_store(buf + L::opp(q) * tcp + x, f[q]);
      } else {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int ex = L::ex(q);
          const int xt = ex == 0 ? x : (ex > 0 ? xp : xm);
          Store<T>::raw_store(buf + L::opp(q) * tcp + xt, f[q]);
        }
      }
    }
    fence_async_smem();
    mbar_arrive(smem_addr(&done[s]));
    if (++s == NST) {
      s = 0;
      ph ^= 1;
    }
  }
}

constexpr int MULTI_STAGES = 3;  // stages of the fused launch (LBMPSM_MULTI_STAGES: 3-5)

template <typename T, int NST>
static cudaError_t multi_set_limits(size_t smem) {
  const void* fns[4] = {(const void*)collide_multi_kernel<D3Q19, T, false, false, NST>,
                        (const void*)collide_multi_kernel<D3Q19, T, false, true, NST>,
                        (const void*)collide_multi_kernel<D3Q19, T, true, false, NST>,
                        (const void*)collide_multi_kernel<D3Q19, T, true, true, NST>};
  for (const void* fn : fns) {
    const cudaError_t e = raise_smem_limit(fn, smem);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T>
static const void* multi_probe_fn(int nst) {
  switch (nst) {
    case 4: return (const void*)collide_multi_kernel<D3Q19, T, true, true, 4>;
    case 5: return (const void*)collide_multi_kernel<D3Q19, T, true, true, 5>;
    default: return (const void*)collide_multi_kernel<D3Q19, T, true, true, 3>;
  }
}

template <typename T>
static cudaError_t multi_prepare(MultiCollide& mc, MultiMember* mem, int sm_count) {
  constexpr int Q = D3Q19::Q;
  // consumers: the widest row, rounded up to whole warps (LBMPSM_MULTI_CONSUMERS
  // asks for more, up to MULTI_MAX_ROW, so that more rows share a tile)
  int smax = 0;
  for (int m = 0; m < mc.nm; ++m) smax = std::max(smax, mem[m].p.g.S[0]);
  if (smax < 1 || smax > MULTI_MAX_ROW) return cudaErrorInvalidValue;
  int tc = (smax + 31) / 32 * 32;
  if (const char* env = std::getenv("LBMPSM_MULTI_CONSUMERS"))
    tc = std::min(MULTI_MAX_ROW, std::max(tc, (std::atoi(env) + 31) / 32 * 32));
  int tcp = 0, total = 0;
  for (int m = 0; m < mc.nm; ++m) {
    const Geom& g = mem[m].p.g;
    int k = std::max(1, tc / g.S[0]);
    k = std::min(k, g.S[1]);
    mem[m].k = k;
    mem[m].tpp = (g.S[1] + k - 1) / k;
    mem[m].ftpp = make_fastdiv((unsigned)mem[m].tpp);
    tcp = std::max(tcp, k * g.P0);
    mc.first[m] = total;
    const long long tiles = (long long)g.S[2] * mem[m].tpp;
    // tile indices stay 32-bit and exact for the multiply-high division
    if (tiles * mem[m].tpp >= (1ll << 32) || total + tiles >= (1ll << 31)) return cudaErrorInvalidValue;
    total += (int)tiles;
  }
  mc.first[mc.nm] = total;
  mc.tcp = (tcp + 7) / 8 * 8;
  const int threads = tc + 32;
  int nst = MULTI_STAGES;
  if (const char* env = std::getenv("LBMPSM_MULTI_STAGES")) nst = std::atoi(env);
  if (nst < 3 || nst > 5) nst = MULTI_STAGES;
  const size_t smem = (size_t)nst * Q * mc.tcp * sizeof(T);
  cudaError_t e = nst == 4 ? multi_set_limits<T, 4>(smem)
                           : (nst == 5 ? multi_set_limits<T, 5>(smem) : multi_set_limits<T, 3>(smem));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, multi_probe_fn<T>(nst), threads,
                                                         smem)) != cudaSuccess)
    return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  mc.pipe.stages = nst;
  mc.pipe.threads = threads;
  mc.pipe.smem = smem;
  mc.pipe.grid = (int)std::min<long long>(total, (long long)per_sm * sm_count);
  return cudaSuccess;
}

cudaError_t prepare_collide_multi(MultiCollide& mc, MultiMember* mem, int storage, int sm_count) {
  if (storage == 0) {
    // FP64: the members' own (row, x-chunk) blocks in turn
    int total = 0;
    for (int m = 0; m < mc.nm; ++m) {
      const Geom& g = mem[m].p.g;
      const long long blocks = (long long)((g.S[0] + 127) / 128) * g.S[1] * g.S[2];
      if (total + blocks >= (1ll << 31)) return cudaErrorInvalidValue;
      mc.first[m] = total;
      total += (int)blocks;
    }
    mc.first[mc.nm] = total;
    return cudaSuccess;
  }
  if (storage == 1) return multi_prepare<float>(mc, mem, sm_count);
  if (storage == 3) return multi_prepare<__nv_bfloat16>(mc, mem, sm_count);
  return multi_prepare<__half>(mc, mem, sm_count);
}

template <typename T, int NST>
static void launch_multi_n(const MultiCollide& mc, int odd, cudaStream_t st) {
  const PipeConfig& c = mc.pipe;
  if (odd) {
    if (mc.any_force)
      collide_multi_kernel<D3Q19, T, true, true, NST><<<c.grid, c.threads, c.smem, st>>>(mc);
    else
      collide_multi_kernel<D3Q19, T, true, false, NST><<<c.grid, c.threads, c.smem, st>>>(mc);
  } else {
    if (mc.any_force)
      collide_multi_kernel<D3Q19, T, false, true, NST><<<c.grid, c.threads, c.smem, st>>>(mc);
    else
      collide_multi_kernel<D3Q19, T, false, false, NST><<<c.grid, c.threads, c.smem, st>>>(mc);
  }
}

template <typename T>
static void launch_multi_t(const MultiCollide& mc, int odd, cudaStream_t st) {
  switch (mc.pipe.stages) {
    case 4: launch_multi_n<T, 4>(mc, odd, st); break;
    case 5: launch_multi_n<T, 5>(mc, odd, st); break;
    default: launch_multi_n<T, 3>(mc, odd, st); break;
  }
}

cudaError_t launch_collide_multi(const MultiCollide& mc, int storage, int odd, cudaStream_t st) {
  if (storage == 0) return launch_collide_f64_multi(mc, odd, st);
  if (mc.pipe.grid <= 0) return cudaSuccess;
  if (storage == 1)
    launch_multi_t<float>(mc, odd, st);
  else if (storage == 3)
    launch_multi_t<__nv_bfloat16>(mc, odd, st);
  else
    launch_multi_t<__half>(mc, odd, st);
  return cudaGetLastError();
}

template <class L, typename T, int NST, int MINB>
static cudaError_t pipe_prepare(const Geom& g, int sm_count, PipeConfig* cfg) {
  const int threads = (g.S[0] + 31) / 32 * 32 + 32;  // consumers + producer warp
  const size_t smem = (size_t)NST * L::Q * g.P0 * sizeof(T);
  cudaError_t e;
  const void* fns[4] = {(const void*)collide_pipe_kernel<L, T, false, false, NST, MINB>,
                        (const void*)collide_pipe_kernel<L, T, false, true, NST, MINB>,
                        (const void*)collide_pipe_kernel<L, T, true, false, NST, MINB>,
                        (const void*)collide_pipe_kernel<L, T, true, true, NST, MINB>};
  for (const void* fn : fns)
    if ((e = raise_smem_limit(fn, smem)) != cudaSuccess) return e;
  int per_sm = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fns[0], threads, smem)) !=
      cudaSuccess)
    return e;
  if (per_sm < 1) return cudaSuccess;  // does not fit: direct kernel
  const long long rows = (long long)g.S[1] * g.S[2];
  const long long grid = std::min<long long>(rows, (long long)per_sm * sm_count);
  cfg->stages = NST;
  cfg->grid = (int)grid;
  cfg->threads = threads;
  cfg->smem = smem;
  cfg->dy = (int)(grid % g.S[1]);
  cfg->dz = (int)(grid / g.S[1]);
  return cudaSuccess;
}

// Blocks per multiprocessor the launch bounds ask for: three for two or three
// stages (72 registers), two for four or five; with 16-bit storage a stage is
// half as large and two or three stages run four blocks (56 registers, a few
// spilled), which the measured 256^3 step favours by 7-10 us.
template <class L, typename T>
static cudaError_t prepare_lowp(const Geom& g, int sm_count, int stages, PipeConfig* cfg) {
  *cfg = PipeConfig{};
  if (g.S[0] > STAGED_MAX_ROW) return cudaSuccess;
  switch (stages) {
    case 0: return cudaSuccess;  // the direct kernel
    case 2: return pipe_prepare<L, T, 2, sizeof(T) == 2 ? 4 : 3>(g, sm_count, cfg);
    case 4: return pipe_prepare<L, T, 4, 2>(g, sm_count, cfg);
    case 5: return pipe_prepare<L, T, 5, 2>(g, sm_count, cfg);
    default: return pipe_prepare<L, T, 3, sizeof(T) == 2 ? 4 : 3>(g, sm_count, cfg);
  }
}

cudaError_t prepare_collide_lowp(const Geom& g, int storage, int sm_count, int stages,
                                 PipeConfig* cfg) {
  if (storage == 1)
    return g.dim == 2 ? prepare_lowp<D2Q9, float>(g, sm_count, stages, cfg)
                      : prepare_lowp<D3Q19, float>(g, sm_count, stages, cfg);
  if (storage == 3)
    return g.dim == 2 ? prepare_lowp<D2Q9, __nv_bfloat16>(g, sm_count, stages, cfg)
                      : prepare_lowp<D3Q19, __nv_bfloat16>(g, sm_count, stages, cfg);
  return g.dim == 2 ? prepare_lowp<D2Q9, __half>(g, sm_count, stages, cfg)
                    : prepare_lowp<D3Q19, __half>(g, sm_count, stages, cfg);
}

template <class L, typename T, int NST, int MINB>
static void launch_pipe(const CollideParams& p, int odd, cudaStream_t st) {
  const PipeConfig& c = p.pipe;
  if (odd) {
    if (p.has_force)
      collide_pipe_kernel<L, T, true, true, NST, MINB><<<c.grid, c.threads, c.smem, st>>>(p);
    else
      collide_pipe_kernel<L, T, true, false, NST, MINB><<<c.grid, c.threads, c.smem, st>>>(p);
  } else {
    if (p.has_force)
      collide_pipe_kernel<L, T, false, true, NST, MINB><<<c.grid, c.threads, c.smem, st>>>(p);
    else
      collide_pipe_kernel<L, T, false, false, NST, MINB><<<c.grid, c.threads, c.smem, st>>>(p);
  }
}

template <class L, typename T>
static cudaError_t launch_lowp(const CollideParams& p, int odd, cudaStream_t st) {
  if (p.pipe.grid > 0) {
    switch (p.pipe.stages) {
      case 2: launch_pipe<L, T, 2, sizeof(T) == 2 ? 4 : 3>(p, odd, st); break;
      case 4: launch_pipe<L, T, 4, 2>(p, odd, st); break;
      case 5: launch_pipe<L, T, 5, 2>(p, odd, st); break;
      default: launch_pipe<L, T, 3, sizeof(T) == 2 ? 4 : 3>(p, odd, st); break;
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

// The project's autotuner for the FP32/FP16 collide: every candidate launch
// shape -- the row pipeline with 3, 2, 4 or 5 stages, each at the blocks per
// multiprocessor its shared memory and registers allow -- runs a few even/odd
// step pairs on p.f (a scratch copy of the populations), timed with CUDA
// events on the stream; the fastest is kept.  The candidates are one template
// (only the stage count and the launch bounds differ), so they round alike
// and the choice changes speed only, never results.  The direct kernel (the
// fallback for rows longer than one staged block) is not a candidate: it
// inlines the same node arithmetic into another kernel, where the compiler's
// multiply-add contraction may round differently.
cudaError_t tune_collide_lowp(CollideParams p, int storage, int sm_count, cudaStream_t st,
                              PipeConfig* best, float* ms_out) {
  const int cand[LBMPSM_TUNE_CANDIDATES] = {3, 2, 4, 5};
  cudaEvent_t e0, e1;
  cudaError_t e = cudaEventCreate(&e0);
  if (e != cudaSuccess) return e;
  if ((e = cudaEventCreate(&e1)) != cudaSuccess) {
    cudaEventDestroy(e0);
    return e;
  }
  float best_ms = 0.0f;
  bool have = false;
  for (int k = 0; k < LBMPSM_TUNE_CANDIDATES; ++k) {
    ms_out[k] = -1.0f;
    PipeConfig c{};
    if (cand[k] > 0) {
      if ((e = prepare_collide_lowp(p.g, storage, sm_count, cand[k], &c)) != cudaSuccess) break;
      if (c.grid == 0) continue;  // this shape does not fit the lattice's rows
    }
    p.pipe = c;
    auto pair = [&]() {
      for (int odd = 0; odd < 2; ++odd)
        if (storage == 1)
          launch_collide_f32(p, odd, st);
        else if (storage == 3)
          launch_collide_bf16(p, odd, st);
        else
          launch_collide_f16(p, odd, st);
    };
    pair();  // warm-up
    cudaEventRecord(e0, st);
    constexpr int REPS = 3;
    for (int r = 0; r < REPS; ++r) pair();
    cudaEventRecord(e1, st);
    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms_out[k] = ms / REPS;
    if (!have || ms_out[k] < best_ms) {
      best_ms = ms_out[k];
      *best = c;
      have = true;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return e;
}

cudaError_t launch_collide_f32(const CollideParams& p, int odd, cudaStream_t st) {
  return p.g.dim == 2 ? launch_lowp<D2Q9, float>(p, odd, st) : launch_lowp<D3Q19, float>(p, odd, st);
}
cudaError_t launch_collide_f16(const CollideParams& p, int odd, cudaStream_t st) {
  return p.g.dim == 2 ? launch_lowp<D2Q9, __half>(p, odd, st)
                      : launch_lowp<D3Q19, __half>(p, odd, st);
}
cudaError_t launch_collide_bf16(const CollideParams& p, int odd, cudaStream_t st) {
  return p.g.dim == 2 ? launch_lowp<D2Q9, __nv_bfloat16>(p, odd, st)
                      : launch_lowp<D3Q19, __nv_bfloat16>(p, odd, st);
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
cudaError_t launch_bc_bf16(const BCParams& p, cudaStream_t st) {
  return launch_bc_lowp<__nv_bfloat16>(p, st);
}

}  // namespace lbmpsm
