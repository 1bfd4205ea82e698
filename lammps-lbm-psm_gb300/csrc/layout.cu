// layout.cu -- population initialisation, conversion between the device
// A-A storage and the reference's FP64 array-of-structures layout, and the
// FP64 global mass/momentum/finite check.
//
// Post-stream population q of node x (what the reference holds in f_curr
// after a step) lives, after an even step, in the opposite slot of the
// upstream node x - e_q, and after an odd step in slot q of x itself.  When
// the upstream node does not exist (array boundary of a non-periodic axis)
// the reference never writes that entry and it keeps the initial
// equilibrium w_q (src/LBM_PSM_BGK_dynamics.cpp:94-99 skips targets outside
// the array).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "lbmpsm_internal.cuh"

namespace lbmpsm {

template <typename T>
__device__ __forceinline__ double load_pop(const void* f, long long loc, int storage, float scale,
                                           double w) {
  (void)sizeof(T);
  if (storage == 0) return static_cast<const double*>(f)[loc];
  if (storage == 1) return w + (double)static_cast<const float*>(f)[loc];
  if (storage == 3) return w + (double)__bfloat162float(static_cast<const __nv_bfloat16*>(f)[loc]);
  return w + (double)(__half2float(static_cast<const __half*>(f)[loc]) / scale);
}

__device__ __forceinline__ void store_pop(void* f, long long loc, int storage, float scale,
                                          double w, double v) {
  if (storage == 0)
    static_cast<double*>(f)[loc] = v;
  else if (storage == 1)
    static_cast<float*>(f)[loc] = (float)(v - w);
  else if (storage == 3)
    static_cast<__nv_bfloat16*>(f)[loc] = __float2bfloat16_rn((float)(v - w));
  else
    static_cast<__half*>(f)[loc] = __float2half_rn((float)(v - w) * scale);
}

template <class L>
__device__ __forceinline__ long long loc_of(const Geom& g, const Nbr& nb, long long n, int q,
                                            int after_odd) {
  const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
  if (!nbr_ok(nb, -cx, -cy, -cz)) return -1;
  if (after_odd) return (long long)q * g.Np + n;
  return (long long)L::opp(q) * g.Np + n + nbr_off(nb, -cx, -cy, -cz);
}

template <class L>
__global__ void init_kernel(Geom g, void* f, int storage, float scale) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.Np) return;
  for (int q = 0; q < L::Q; ++q) {
    const long long loc = (long long)q * g.Np + n;
    if (storage == 0)
      static_cast<double*>(f)[loc] = L::w(q);  // feq(rho = 1, u = 0) = w_q
    else if (storage == 1)
      static_cast<float*>(f)[loc] = 0.0f;
    else if (storage == 3)
      static_cast<__nv_bfloat16*>(f)[loc] = __float2bfloat16_rn(0.0f);
    else
      static_cast<__half*>(f)[loc] = __float2half_rn(0.0f);
  }
}

cudaError_t launch_init_populations(const Geom& g, void* f, int storage, float scale16,
                                    cudaStream_t st) {
  const unsigned blocks = (unsigned)((g.Np + 255) / 256);
  if (g.dim == 2)
    init_kernel<D2Q9><<<blocks, 256, 0, st>>>(g, f, storage, scale16);
  else
    init_kernel<D3Q19><<<blocks, 256, 0, st>>>(g, f, storage, scale16);
  return cudaGetLastError();
}

// One thread per node of the reference local array (halo included); periodic
// halo nodes read their periodic twin, as after the reference's exchange.
template <class L>
__global__ void get_pop_kernel(Geom g, const void* f, int storage, int after_odd, float scale,
                               double* out) {
  const long long total = (long long)g.L[0] * g.L[1] * g.L[2];
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= total) return;
  const int k = (int)(r % g.L[2]);
  const int j = (int)((r / g.L[2]) % g.L[1]);
  const int i = (int)(r / ((long long)g.L[2] * g.L[1]));
  const int h[3] = {i, j, k};
  int s[3];
  for (int d = 0; d < 3; ++d) {
    if (g.off[d] == 1) {
      s[d] = h[d] - 1;
      if (s[d] < 0) s[d] = g.S[d] - 1;
      if (s[d] >= g.S[d]) s[d] = 0;
    } else {
      s[d] = h[d];
    }
  }
  const long long n = node_index(g, s[0], s[1], s[2]);
  const Nbr nb = make_nbr(g, s[0], s[1], s[2]);
  for (int q = 0; q < L::Q; ++q) {
    const long long loc = loc_of<L>(g, nb, n, q, after_odd);
    out[r * L::Q + q] = loc >= 0 ? load_pop<int>(f, loc, storage, scale, L::w(q)) : L::w(q);
  }
}

template <class L>
__global__ void set_pop_kernel(Geom g, void* f, int storage, int after_odd, float scale,
                               const double* in) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.N) return;
  const int sx = (int)(n % g.P0);
  const int sy = (int)((n / g.P0) % g.S[1]);
  const int sz = (int)(n / ((long long)g.P0 * g.S[1]));
  if (sx >= g.S[0]) return;  // x padding
  const long long r = ((long long)(sx + g.off[0]) * g.L[1] + (sy + g.off[1])) * g.L[2] + (sz + g.off[2]);
  const Nbr nb = make_nbr(g, sx, sy, sz);
  for (int q = 0; q < L::Q; ++q) {
    const long long loc = loc_of<L>(g, nb, n, q, after_odd);
    if (loc >= 0) store_pop(f, loc, storage, scale, L::w(q), in[r * L::Q + q]);
  }
}

cudaError_t launch_get_populations(const Geom& g, const void* f, int storage, int after_odd,
                                   float scale16, double* out_ref, cudaStream_t st) {
  const long long total = (long long)g.L[0] * g.L[1] * g.L[2];
  const unsigned blocks = (unsigned)((total + 255) / 256);
  if (g.dim == 2)
    get_pop_kernel<D2Q9><<<blocks, 256, 0, st>>>(g, f, storage, after_odd, scale16, out_ref);
  else
    get_pop_kernel<D3Q19><<<blocks, 256, 0, st>>>(g, f, storage, after_odd, scale16, out_ref);
  return cudaGetLastError();
}

cudaError_t launch_set_populations(const Geom& g, void* f, int storage, int after_odd,
                                   float scale16, const double* in_ref, cudaStream_t st) {
  const unsigned blocks = (unsigned)((g.N + 255) / 256);
  if (g.dim == 2)
    set_pop_kernel<D2Q9><<<blocks, 256, 0, st>>>(g, f, storage, after_odd, scale16, in_ref);
  else
    set_pop_kernel<D3Q19><<<blocks, 256, 0, st>>>(g, f, storage, after_odd, scale16, in_ref);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ check
constexpr int CHECK_THREADS = 256;
constexpr int CHECK_BLOCKS = 1024;

// Error-free transformation a + b = s + e (Knuth's TwoSum, no contraction).
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fadd_rn(s, -a);
  e = __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bb)), __fadd_rn(b, -bb));
}

// Blocks walk x-rows with 32-bit index arithmetic (64-bit integer division
// is emulated and slow).  FP64 storage sums the populations in FP64.  FP32 /
// FP16 / BF16 storage sums each node's deviations g = f - w in FP32 and adds the
// node sums into double-float accumulators on the FP32 pipe; the weights add
// up to exactly 1 per node (mass = nodes + sum g) and to 0 in every momentum
// component.
template <class L, bool F64>
__global__ void __launch_bounds__(CHECK_THREADS) check_partial_kernel(Geom g, const void* f,
                                                                       int storage, int after_odd,
                                                                       float scale, double* partial,
                                                                       int* status) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
  unsigned nodes = 0;
  bool bad = false;
  const float inv_scale = 1.0f / scale;
  const int R = g.S[1] * g.S[2];
  for (int r = blockIdx.x; r < R; r += gridDim.x) {
    const int sy = r % g.S[1], sz = r / g.S[1];
    for (int sx = threadIdx.x; sx < g.S[0]; sx += blockDim.x) {
      const long long n = node_index(g, sx, sy, sz);
      const Nbr nb = make_nbr(g, sx, sy, sz);
      if (F64) {
        for (int q = 0; q < L::Q; ++q) {
          const long long loc = loc_of<L>(g, nb, n, q, after_odd);
          const double v = loc >= 0 ? static_cast<const double*>(f)[loc] : L::w(q);
          if (!isfinite(v)) bad = true;
          acc[0] += v;
          acc[1] += v * L::ex(q);
          acc[2] += v * L::ey(q);
          acc[3] += v * L::ez(q);
        }
      } else {
        float ns[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int q = 0; q < L::Q; ++q) {
          const long long loc = loc_of<L>(g, nb, n, q, after_odd);
          float v = 0.0f;
          if (loc >= 0)
            v = storage == 1   ? static_cast<const float*>(f)[loc]
                : storage == 3 ? __bfloat162float(static_cast<const __nv_bfloat16*>(f)[loc])
                               : __half2float(static_cast<const __half*>(f)[loc]) * inv_scale;
          if (!isfinite(v)) bad = true;
          ns[0] += v;
          if (L::ex(q)) ns[1] += L::ex(q) > 0 ? v : -v;
          if (L::ey(q)) ns[2] += L::ey(q) > 0 ? v : -v;
          if (L::ez(q)) ns[3] += L::ez(q) > 0 ? v : -v;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          float sv, e;
          two_sum_f(hi[k], ns[k], sv, e);
          hi[k] = sv;
          lo[k] = __fadd_rn(lo[k], e);
        }
        ++nodes;
      }
    }
  }
  if (!F64) {
    acc[0] = (double)hi[0] + (double)lo[0] + (double)nodes;
    for (int k = 1; k < 4; ++k) acc[k] = (double)hi[k] + (double)lo[k];
  }
  if (bad) atomicOr(status, STATUS_NONFINITE);
  for (int k = 0; k < 4; ++k)
    for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
  __shared__ double part[CHECK_THREADS / 32][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int k = 0; k < 4; ++k) part[warp][k] = acc[k];
  __syncthreads();
  if (threadIdx.x < 4) {
    double s = 0.0;
    for (int w = 0; w < CHECK_THREADS / 32; ++w) s += part[w][threadIdx.x];
    partial[4 * blockIdx.x + threadIdx.x] = s;
  }
}

__global__ void check_final_kernel(const double* partial, int nblocks, double* acc4) {
  if (threadIdx.x < 4) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += partial[4 * b + threadIdx.x];
    acc4[threadIdx.x] = s;
  }
}

// acc4 must have room for 4 + 4*CHECK_BLOCKS doubles (partials after the sums).
cudaError_t launch_check(const Geom& g, const void* f, int storage, int after_odd, float scale16,
                         double* acc4, int* status, cudaStream_t st) {
  double* partial = acc4 + 4;
  if (g.dim == 2) {
    if (storage == 0)
      check_partial_kernel<D2Q9, true><<<CHECK_BLOCKS, CHECK_THREADS, 0, st>>>(
          g, f, storage, after_odd, scale16, partial, status);
    else
      check_partial_kernel<D2Q9, false><<<CHECK_BLOCKS, CHECK_THREADS, 0, st>>>(
          g, f, storage, after_odd, scale16, partial, status);
  } else {
    if (storage == 0)
      check_partial_kernel<D3Q19, true><<<CHECK_BLOCKS, CHECK_THREADS, 0, st>>>(
          g, f, storage, after_odd, scale16, partial, status);
    else
      check_partial_kernel<D3Q19, false><<<CHECK_BLOCKS, CHECK_THREADS, 0, st>>>(
          g, f, storage, after_odd, scale16, partial, status);
  }
  check_final_kernel<<<1, 32, 0, st>>>(partial, CHECK_BLOCKS, acc4);
  return cudaGetLastError();
}

}  // namespace lbmpsm
