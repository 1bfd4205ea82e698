// adjoint.cu -- discrete adjoint and tangent of the FP64 collide-stream-PSM
// step on a fully periodic lattice with the particles held in place.
//
// Forward step (one node, pre-collision populations f, table weights B_s and
// solid velocities us_s; compute_macro_values + collisionAndStream,
// src/LBM_PSM_BGK_dynamics.cpp:48-109, src/LBM_PSM_BGK_dynamics.h:40-114,
// feq / F_iq src/LBM_PSM_dynamics.h:43-116), in exact arithmetic:
//
//   rho = sum f, m = sum f e, j = m + F/2, u = j / rho
//   C_q = (1-w) f_q + (w - Bt) feq_q(rho, u) + sum_s B_s feq_q(rho, us_s) + (1 - w/2) g_q(u)
//   g_q = w_q [3 (e_q - u).F + 9 (e_q.u)(e_q.F)]             (unscaled Guo term)
//   f_{t+1, q}(x + e_q) = C_q(x)                              (streaming)
//   slot force (add_Fhyd, src/LBM_PSM_lattice.cpp:355-363):
//   -B_s sum_q Omega_s,q e_q = B_s (m + (1-w) F/2 - rho us_s)
//
// Objective: J = sum_t c_t sum_nodes sum_s cw_s d . (slot force), where cw_s
// counts the images of the slot's particle whose reduction box holds the
// node (calculateHydrodynamicInteractions, src/LBM_PSM_exchangeParticleData.cpp:172-244)
// and c_t = forceFactor / M inside the averaging window, 0 outside.
//
// The reverse step pulls the adjoint of the next step's pre-collision
// populations, mu_q(x) = lambda_{t+1,q}(x + e_q), and applies the transposed
// node Jacobian through moments of w_q mu_q (M0, M1_a, M2_ab), so that every
// contraction sum_q mu_q dC_q/d(.) costs a few FP64 operations per node.
// The tangent step pushes dC along a direction (dtau, dF, dx).  Centre
// derivatives enter through the solid fractions: the central difference of
// calcSolidFraction's sub-cell count (src/LBM_PSM_exchangeParticleData.cpp:116-169)
// at step h, computed exactly with the reference's FP64 operations.
#include "lbmpsm_internal.cuh"

namespace lbmpsm {

namespace {

constexpr int ADJ_THREADS = 128;

// Weights of the two slots and their derivatives (BGK weighting B = eps, or
// Noble-Torczynski B = eps (tau-1/2) / ((1-eps) + tau-1/2); renormalised to
// sum 1 when the sum exceeds 1, as in collisionAndStream :90-95).
struct SlotWeights {
  double B[2];
  double dBde[2][2];  // dB_r / deps_k
  double dBdtau[2];
};

__device__ __forceinline__ void slot_weights(double e0, double e1, bool occ0, bool occ1,
                                             int weighting, double tau, SlotWeights& w) {
  const double e[2] = {occ0 ? e0 : 0.0, occ1 ? e1 : 0.0};
  double b[2], db[2], dbt[2];
  const double tm = tau - 0.5;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (weighting == 1) {
      const double den = (1.0 - e[k]) + tm;
      b[k] = e[k] * tm / den;
      db[k] = tm * (1.0 + tm) / (den * den);
      dbt[k] = e[k] * (1.0 - e[k]) / (den * den);
    } else {
      b[k] = e[k];
      db[k] = 1.0;
      dbt[k] = 0.0;
    }
  }
  const double s = b[0] + b[1];
  double J[2][2];
  if (s > 1.0) {
    const double is2 = 1.0 / (s * s);
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      w.B[r] = b[r] / s;
#pragma unroll
      for (int k = 0; k < 2; ++k) J[r][k] = ((r == k ? s : 0.0) - b[r]) * is2;
    }
  } else {
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      w.B[r] = b[r];
#pragma unroll
      for (int k = 0; k < 2; ++k) J[r][k] = r == k ? 1.0 : 0.0;
    }
  }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    w.dBde[r][0] = J[r][0] * db[0];
    w.dBde[r][1] = J[r][1] * db[1];
    w.dBdtau[r] = J[r][0] * dbt[0] + J[r][1] * dbt[1];
  }
}

// Moments of v_q = w_q mu_q: M0 = sum v, M1_a = sum v e_a,
// M2 = sum v e_a e_b in the order xx, yy, zz, xy, xz, yz.
template <class L>
__device__ __forceinline__ void moments(const double* mu, double& M0, double M1[3],
                                        double M2[6]) {
  M0 = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) M1[a] = 0.0;
#pragma unroll
  for (int a = 0; a < 6; ++a) M2[a] = 0.0;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    constexpr int dummy = 0;
    (void)dummy;
    const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    const double v = L::w(q) * mu[q];
    M0 += v;
    if (cx) M1[0] += cx > 0 ? v : -v;
    if (cy) M1[1] += cy > 0 ? v : -v;
    if (cz) M1[2] += cz > 0 ? v : -v;
    if (cx) M2[0] += v;
    if (cy) M2[1] += v;
    if (cz) M2[2] += v;
    if (cx && cy) M2[3] += cx * cy > 0 ? v : -v;
    if (cx && cz) M2[4] += cx * cz > 0 ? v : -v;
    if (cy && cz) M2[5] += cy * cz > 0 ? v : -v;
  }
}

__device__ __forceinline__ void m2_times(const double M2[6], const double a[3], double out[3]) {
  out[0] = M2[0] * a[0] + M2[3] * a[1] + M2[4] * a[2];
  out[1] = M2[3] * a[0] + M2[1] * a[1] + M2[5] * a[2];
  out[2] = M2[4] * a[0] + M2[5] * a[1] + M2[2] * a[2];
}

__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

template <class L, int q>
__device__ __forceinline__ double edot_c(const double v[3]) {
  double s = 0.0;
  if (L::ex(q)) s += L::ex(q) > 0 ? v[0] : -v[0];
  if (L::ey(q)) s += L::ey(q) > 0 ? v[1] : -v[1];
  if (L::ez(q)) s += L::ez(q) > 0 ? v[2] : -v[2];
  return s;
}

template <class L, int q>
struct Unroll {
  template <class Fn>
  __device__ __forceinline__ static void run(Fn& fn) {
    fn.template apply<q>();
    Unroll<L, q + 1>::run(fn);
  }
};
template <class L>
struct Unroll<L, L::Q> {
  template <class Fn>
  __device__ __forceinline__ static void run(Fn&) {}
};

// the pre-collision populations of node n in A-A storage, as the FP64
// collide kernel reads them
template <class L>
__device__ __forceinline__ void load_state(const double* F, long long Np, long long n,
                                           const Nbr& nb, int odd, double* f) {
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    if (!odd)
      f[q] = F[q * Np + n];
    else
      f[q] = F[L::opp(q) * Np + n + nbr_off(nb, -cx, -cy, -cz)];
  }
}

// One node's slots as the sweeps see them.
struct NodeSlots {
  bool live[2];     // slot has a particle (table) or an entering one (band)
  bool band;
  double B[2];
  double us[2][3];
  double cw[2];
  SlotWeights w;
};

__device__ __forceinline__ void node_slots(const AdjParams& p, long long n, NodeSlots& s) {
  const uint8_t flag = p.tab.flag[n];
  const uint8_t band = p.an.band[n];
  s.band = band != 0;
  s.live[0] = s.live[1] = false;
  s.B[0] = s.B[1] = 0.0;
  s.cw[0] = s.cw[1] = 0.0;
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) s.us[k][c] = 0.0;
  if (!flag && !band) return;
  int2 id = make_int2(0, 0);
  double2 e = make_double2(0.0, 0.0);
  if (flag) {
    id = p.tab.ids[n];
    e = p.tab.eps[n];
  }
  const bool occ0 = id.x > 0, occ1 = id.y > 0;
  slot_weights(e.x, e.y, occ0, occ1, p.weighting, p.bp.tau, s.w);
  const int2 cw = p.an.cw[n];
  const int2 et = band ? p.an.tag[n] : make_int2(0, 0);
  const bool occ[2] = {occ0, occ1};
  const int etag[2] = {et.x, et.y};
  const int cwk[2] = {cw.x, cw.y};
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (occ[k]) {
      s.live[k] = true;
      s.B[k] = s.w.B[k];
#pragma unroll
      for (int c = 0; c < 3; ++c) s.us[k][c] = p.tab.us[6 * n + 3 * k + c];
      s.cw[k] = (double)cwk[k];
    } else if (etag[k] > 0) {
      s.live[k] = true;
#pragma unroll
      for (int c = 0; c < 3; ++c) s.us[k][c] = p.an.us[6 * n + 3 * k + c];
      s.cw[k] = (double)cwk[k];
    }
  }
}

// deterministic block sum of ADJ_PART values into this block's slot
__device__ __forceinline__ void block_accumulate(double (&v)[ADJ_PART], double* part) {
  __shared__ double red[ADJ_THREADS / 32][ADJ_PART];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < ADJ_PART; ++k) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[wid][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < ADJ_PART) {
    double x = 0.0;
#pragma unroll
    for (int w = 0; w < ADJ_THREADS / 32; ++w) x += red[w][threadIdx.x];
    part[(long long)blockIdx.x * ADJ_PART + threadIdx.x] += x;
  }
}

// ------------------------------------------------------------ reverse step
template <class L>
struct AdjQ {
  // inputs
  const double* mu;
  double omBt, omw, inv_rho, uAu;
  double Aj[3], Au[3], cB[2], dus[2];
  double base;  // (1-w) mu term is per q; base = A_rho + sum_s B_s A_s - uAu/rho + drag const
  double coef;  // drag coefficient of d.e_q
  const double* d;
  double* out;
  template <int q>
  __device__ __forceinline__ void apply() {
    const double ej = edot_c<L, q>(Aj);
    const double eAu = edot_c<L, q>(Au);
    const double de = edot_c<L, q>(d);
    out[q] = omw * mu[q] + omBt * ej + base + eAu * inv_rho + coef * de;
  }
};

template <class L>
__global__ void __launch_bounds__(ADJ_THREADS) adj_step_kernel(AdjParams p) {
  constexpr int Q = L::Q;
  const Geom& g = p.g;
  const int xblocks = (g.S[0] + ADJ_THREADS - 1) / ADJ_THREADS;
  const int row = blockIdx.x / xblocks;
  const int sx = (blockIdx.x - row * xblocks) * ADJ_THREADS + threadIdx.x;
  double acc[ADJ_PART] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (sx < g.S[0]) {
    const int sy = row % g.S[1];
    const int sz = row / g.S[1];
    const long long n = node_index(g, sx, sy, sz);
    const Nbr nb = make_nbr(g, sx, sy, sz);
    const long long Np = g.Np;
    const BoxParams& bp = p.bp;
    const double omega = bp.omega;
    const double F[3] = {bp.F[0], bp.F[1], bp.F[2]};
    double f[Q], mu[Q];
    load_state<L>(p.state, Np, n, nb, p.odd, f);
#pragma unroll
    for (int q = 0; q < Q; ++q)
      mu[q] = p.lin[q * Np + n + nbr_off(nb, L::ex(q), L::ey(q), L::ez(q))];
    double rho = 0.0, m[3] = {0.0, 0.0, 0.0}, smf = 0.0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      rho += f[q];
      smf += mu[q] * f[q];
      if (L::ex(q)) m[0] += L::ex(q) > 0 ? f[q] : -f[q];
      if (L::ey(q)) m[1] += L::ey(q) > 0 ? f[q] : -f[q];
      if (L::ez(q)) m[2] += L::ez(q) > 0 ? f[q] : -f[q];
    }
    const double inv_rho = 1.0 / rho;
    double u[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) u[a] = (m[a] + 0.5 * F[a]) * inv_rho;
    double M0, M1[3], M2[6];
    moments<L>(mu, M0, M1, M2);
    const double usq = dot3(u, u);
    double M2u[3], M2F[3];
    m2_times(M2, u, M2u);
    m2_times(M2, F, M2F);
    const double uM2u = dot3(u, M2u);
    const double smfeq = rho * (M0 * (1.0 - 1.5 * usq) + 3.0 * dot3(u, M1) + 4.5 * uM2u);
    const double A_rho = M0 * (1.0 + 1.5 * usq) - 4.5 * uM2u;
    double Aj[3], Au[3];
    const double gp = 1.0 - 0.5 * omega;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      Aj[a] = 3.0 * M1[a] + 9.0 * M2u[a] - 3.0 * u[a] * M0;
      Au[a] = gp * (-3.0 * F[a] * M0 + 9.0 * M2F[a]);
    }
    const double smg = 3.0 * (dot3(M1, F) - M0 * dot3(u, F)) + 9.0 * dot3(u, M2F);
    const double d[3] = {p.d[0], p.d[1], p.d[2]};
    const double dm = dot3(d, m), dF = dot3(d, F);

    NodeSlots sl;
    node_slots(p, n, sl);
    double sumBAs = 0.0, coef = 0.0, dconst = 0.0, Bt = 0.0, sum_cB = 0.0, gtauB = 0.0;
    double beta[2] = {0.0, 0.0};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (!sl.live[k]) continue;
      const double* vs = sl.us[k];
      double M2v[3];
      m2_times(M2, vs, M2v);
      const double As = M0 * (1.0 - 1.5 * dot3(vs, vs)) + 3.0 * dot3(vs, M1) + 4.5 * dot3(vs, M2v);
      const double dvs = dot3(d, vs);
      const double cB = p.c * sl.cw[k] * sl.B[k];
      sumBAs += sl.B[k] * As;
      Bt += sl.B[k];
      coef += cB;
      dconst -= cB * dvs;
      sum_cB += cB;
      beta[k] = rho * As - smfeq +
                p.c * sl.cw[k] * (dm + (1.0 - omega) * dF * 0.5 - rho * dvs);
    }
    if (p.weighting == 1) gtauB = beta[0] * sl.w.dBdtau[0] + beta[1] * sl.w.dBdtau[1];
    if (sl.band) {
      p.an.sigma[2 * n] += beta[0];
      p.an.sigma[2 * n + 1] += beta[1];
    }
    AdjQ<L> fn;
    fn.mu = mu;
    fn.omw = 1.0 - omega;
    fn.omBt = omega - Bt;
    fn.inv_rho = inv_rho;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      fn.Aj[a] = Aj[a];
      fn.Au[a] = Au[a];
    }
    fn.base = (omega - Bt) * A_rho + sumBAs - dot3(u, Au) * inv_rho + dconst;
    fn.coef = coef;
    fn.d = d;
    double out[Q];
    fn.out = out;
    Unroll<L, 0>::run(fn);
#pragma unroll
    for (int q = 0; q < Q; ++q) p.lout[q * Np + n] = out[q];

    acc[0] = smfeq - smf - 0.5 * smg - sum_cB * dF * 0.5;
    acc[1] = gtauB;
#pragma unroll
    for (int a = 0; a < 3; ++a)
      acc[2 + a] = (omega - Bt) * Aj[a] * 0.5 + gp * Aj[a] + Au[a] * (0.5 * inv_rho) +
                   sum_cB * (1.0 - omega) * d[a] * 0.5;
  }
  block_accumulate(acc, p.part);
}

// ------------------------------------------------------------ tangent step
template <class L>
__global__ void __launch_bounds__(ADJ_THREADS) tan_step_kernel(AdjParams p) {
  constexpr int Q = L::Q;
  const Geom& g = p.g;
  const int xblocks = (g.S[0] + ADJ_THREADS - 1) / ADJ_THREADS;
  const int row = blockIdx.x / xblocks;
  const int sx = (blockIdx.x - row * xblocks) * ADJ_THREADS + threadIdx.x;
  double acc[ADJ_PART] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (sx < g.S[0]) {
    const int sy = row % g.S[1];
    const int sz = row / g.S[1];
    const long long n = node_index(g, sx, sy, sz);
    const Nbr nb = make_nbr(g, sx, sy, sz);
    const long long Np = g.Np;
    const BoxParams& bp = p.bp;
    const double omega = bp.omega, domega = p.domega;
    const double F[3] = {bp.F[0], bp.F[1], bp.F[2]};
    const double dFv[3] = {p.dF[0], p.dF[1], p.dF[2]};
    double f[Q], fd[Q];
    load_state<L>(p.state, Np, n, nb, p.odd, f);
#pragma unroll
    for (int q = 0; q < Q; ++q) fd[q] = p.lin[q * Np + n];
    double rho = 0.0, rhod = 0.0, m[3] = {0.0, 0.0, 0.0}, md[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      rho += f[q];
      rhod += fd[q];
      if (L::ex(q)) { m[0] += L::ex(q) > 0 ? f[q] : -f[q]; md[0] += L::ex(q) > 0 ? fd[q] : -fd[q]; }
      if (L::ey(q)) { m[1] += L::ey(q) > 0 ? f[q] : -f[q]; md[1] += L::ey(q) > 0 ? fd[q] : -fd[q]; }
      if (L::ez(q)) { m[2] += L::ez(q) > 0 ? f[q] : -f[q]; md[2] += L::ez(q) > 0 ? fd[q] : -fd[q]; }
    }
    const double inv_rho = 1.0 / rho;
    double u[3], jd[3], ud[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      u[a] = (m[a] + 0.5 * F[a]) * inv_rho;
      jd[a] = md[a] + 0.5 * dFv[a];
      ud[a] = (jd[a] - u[a] * rhod) * inv_rho;
    }
    const double usq = dot3(u, u);
    const double uF = dot3(u, F), udF = dot3(u, dFv), ujd = dot3(u, jd), Fud = dot3(F, ud);

    NodeSlots sl;
    node_slots(p, n, sl);
    double Bd[2] = {0.0, 0.0};
    if (sl.live[0] || sl.live[1]) {
      const double ed0 = sl.band ? p.an.edot[2 * n] : 0.0;
      const double ed1 = sl.band ? p.an.edot[2 * n + 1] : 0.0;
#pragma unroll
      for (int k = 0; k < 2; ++k)
        Bd[k] = sl.w.dBde[k][0] * ed0 + sl.w.dBde[k][1] * ed1 + sl.w.dBdtau[k] * p.dtau;
    }
    const double Bt = sl.B[0] + sl.B[1], Btd = Bd[0] + Bd[1];
    const double gp = 1.0 - 0.5 * omega;
    const double hs[2] = {1.5 * dot3(sl.us[0], sl.us[0]), 1.5 * dot3(sl.us[1], sl.us[1])};
    const double rr = rhod * inv_rho;
    double out[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
      const double w = L::w(q);
      const double eu = cx * u[0] + cy * u[1] + cz * u[2];
      const double ejd = cx * jd[0] + cy * jd[1] + cz * jd[2];
      const double eF = cx * F[0] + cy * F[1] + cz * F[2];
      const double eud = cx * ud[0] + cy * ud[1] + cz * ud[2];
      const double edF = cx * dFv[0] + cy * dFv[1] + cz * dFv[2];
      const double feq = rho * w * (1.0 + 3.0 * eu + 4.5 * eu * eu - 1.5 * usq);
      const double feqd = w * (rhod * (1.0 - 4.5 * eu * eu + 1.5 * usq) + 3.0 * ejd +
                               9.0 * eu * ejd - 3.0 * ujd);
      const double gq = w * (3.0 * (eF - uF) + 9.0 * eu * eF);
      const double gqd = w * (-3.0 * Fud + 9.0 * eF * eud + 3.0 * (edF - udF) + 9.0 * eu * edF);
      double c = (1.0 - omega) * fd[q] - domega * f[q] + (domega - Btd) * feq +
                 (omega - Bt) * feqd - 0.5 * domega * gq + gp * gqd;
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        if (!sl.live[k]) continue;
        const double evs = cx * sl.us[k][0] + cy * sl.us[k][1] + cz * sl.us[k][2];
        const double fs = rho * w * (1.0 + 3.0 * evs + 4.5 * evs * evs - hs[k]);
        c += Bd[k] * fs + sl.B[k] * fs * rr;
      }
      out[q] = c;
    }
#pragma unroll
    for (int q = 0; q < Q; ++q)
      p.lout[q * Np + n + nbr_off(nb, L::ex(q), L::ey(q), L::ez(q))] = out[q];

    const double d[3] = {p.d[0], p.d[1], p.d[2]};
    const double dm = dot3(d, m), dmd = dot3(d, md), dF = dot3(d, F), ddF = dot3(d, dFv);
    double dJ = 0.0;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (!sl.live[k]) continue;
      const double dvs = dot3(d, sl.us[k]);
      const double base = dm + (1.0 - omega) * dF * 0.5 - rho * dvs;
      dJ += p.c * sl.cw[k] *
            (Bd[k] * base +
             sl.B[k] * (dmd - domega * dF * 0.5 + (1.0 - omega) * ddF * 0.5 - rhod * dvs));
    }
    acc[0] = dJ;
  }
  block_accumulate(acc, p.part);
}

// ------------------------------------------------------- entries and weights
__global__ void adj_entries_kernel(AdjSetup s) {
  const Geom& g = s.g;
  const long long total = (long long)g.S[0] * g.S[1] * g.S[2];
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int sx = (int)(idx % g.S[0]);
  const int sy = (int)((idx / g.S[0]) % g.S[1]);
  const int sz = (int)(idx / ((long long)g.S[0] * g.S[1]));
  const long long n = node_index(g, sx, sy, sz);
  const int2 id = s.tab.ids[n];
  const bool occ[2] = {id.x > 0, id.y > 0};
  int tag[2] = {occ[0] ? id.x : 0, occ[1] ? id.y : 0};
  double us[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  bool band = false;
  int seen[4];
  int nseen = 0;
  int status = 0;
  const int hx = sx + g.off[0], hy = sy + g.off[1], hz = sz + g.off[2];
  const int cell = ((sz / s.cb[2]) * s.C[1] + sy / s.cb[1]) * s.C[0] + sx / s.cb[0];
  const int off = s.cell_off[cell], cnt = s.cell_count[cell];
  for (int k = 0; k < cnt; ++k) {
    const Img& im = s.img[s.list[off + k]];
    if (!im.valid) continue;
    if (sx < im.lo[0] || sx >= im.hi[0] || sy < im.lo[1] || sy >= im.hi[1] || sz < im.lo[2] ||
        sz >= im.hi[2])
      continue;
    const double dx = (double)hx - im.xl[0];
    const double dy = (double)hy - im.xl[1];
    const double dz = (double)hz - im.xl[2];
    const double dist = dx * dx + dy * dy + dz * dz;
    const double rl = fmax(im.r - s.h0 - 2.0 * s.hl, 0.0), rh = im.r + s.h0 + 2.0 * s.hl;
    if (dist < rl * rl || dist > rh * rh) continue;
    band = true;
    const int t = im.tag;
    for (int j = 0; j < nseen; ++j)
      if (seen[j] == t) status |= STATUS_ADJ_SAME_TAG;
    if (nseen < 4) seen[nseen++] = t;
    if ((occ[0] && tag[0] == t) || (occ[1] && tag[1] == t)) continue;
    // an entering particle takes the first empty slot (setParticle, src/LBM_PSM_lattice.cpp:257-330)
    int slot = -1;
    if (tag[0] == 0 || tag[0] == t) {
      slot = 0;
    } else if (tag[1] == 0 || tag[1] == t) {
      slot = 1;
    } else {
      status |= STATUS_ADJ_CROWDED;
    }
    if (slot >= 0 && tag[slot] == 0) {
      tag[slot] = t;
      // node velocity u = uT + omega x (node - x_l) (src/LBM_PSM_exchangeParticleData.cpp:83-89)
      us[3 * slot + 0] = im.uT[0] + im.om[1] * dz - im.om[2] * dy;
      us[3 * slot + 1] = im.uT[1] + im.om[2] * dx - im.om[0] * dz;
      us[3 * slot + 2] = im.uT[2] + im.om[0] * dy - im.om[1] * dx;
    }
  }
  int cw[2] = {0, 0};
  if (tag[0] > 0 || tag[1] > 0) {
    for (int k = 0; k < cnt; ++k) {
      const Img& im = s.img[s.list[off + k]];
      if (!im.valid) continue;
      if (hx < im.rlo[0] || hx >= im.rhi[0] || hy < im.rlo[1] || hy >= im.rhi[1] ||
          hz < im.rlo[2] || hz >= im.rhi[2])
        continue;
      // the reduction's tag match: slot 1 first, then slot 2
      if (im.tag == tag[0])
        ++cw[0];
      else if (im.tag == tag[1])
        ++cw[1];
    }
  }
  s.an.band[n] = band ? 1 : 0;
  s.an.tag[n] = make_int2(tag[0], tag[1]);
  s.an.cw[n] = make_int2(cw[0], cw[1]);
  if (band)
    for (int c = 0; c < 6; ++c) s.an.us[6 * n + c] = us[c];
  if (status) atomicOr(s.status, status);
}

// calcSolidFraction (src/LBM_PSM_exchangeParticleData.cpp:116-169) with the
// reference's FP64 operations, none contracted.
__device__ double eps_exact(int dim, int i, int j, int k, const double xl[3], double r,
                            double h0) {
  const int slices = 10;
  const double width = 1.0 / ((double)slices);
  const double fraction = dim == 3 ? 1.0 / ((double)(slices * slices * slices))
                                   : 1.0 / ((double)(slices * slices));
  const double dx = (double)i - xl[0];
  const double dy = (double)j - xl[1];
  const double dz = (double)k - xl[2];
  const double dist = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  const double rP = r + h0;
  if (dist > __dmul_rn(rP, rP)) return 0.0;
  const double rM = r - h0;
  if (dist < __dmul_rn(rM, rM)) return 1.0;
  const double rSq = __dmul_rn(r, r);
  double sx[10], sy[10], sz[10];
#pragma unroll
  for (int m = 0; m < 10; ++m) {
    const double delta = __dadd_rn(-0.5, __dmul_rn(__dadd_rn((double)m, 0.5), width));
    const double a = dx + delta, b = dy + delta, c = dz + delta;
    sx[m] = __dmul_rn(a, a);
    sy[m] = __dmul_rn(b, b);
    sz[m] = __dmul_rn(c, c);
  }
  int cnt = 0;
  if (dim == 2) {
    for (int a = 0; a < 10; ++a)
#pragma unroll
      for (int b = 0; b < 10; ++b) cnt += (sx[a] + sy[b] < rSq) ? 1 : 0;
  } else {
    for (int a = 0; a < 10; ++a)
      for (int b = 0; b < 10; ++b) {
        const double s2 = sx[a] + sy[b];
#pragma unroll
        for (int c = 0; c < 10; ++c) cnt += (s2 + sz[c] < rSq) ? 1 : 0;
      }
  }
  return fraction * ((double)cnt);
}

// lattice-local centre on one rank (src/LBM_PSM_exchangeParticleData.cpp:31-37)
__device__ __forceinline__ double local_centre_of(double x, double origin, double dx) {
  const double g = (x - origin) / dx;
  return g - ((0 - ((double)0 * 2.0 * (double)1)) - 1);
}

constexpr int CEN_THREADS = 256;

// One block per image: the central difference of its solid fraction at
// every surface node of its map box, for each axis; the adjoint contracts it
// with the accumulated dJ/dB, the tangent stores the rate along xdot.
__global__ void __launch_bounds__(CEN_THREADS) adj_centre_kernel(AdjCentre c) {
  const int i = blockIdx.x;
  const Img& im = c.img[i];
  const Geom& g = c.g;
  double acc[3] = {0.0, 0.0, 0.0};
  if (im.valid) {
    double xlp[3], xlm[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      xlp[a] = local_centre_of(c.x[3 * i + a] + c.h, c.origin[a], c.dx);
      xlm[a] = local_centre_of(c.x[3 * i + a] - c.h, c.origin[a], c.dx);
    }
    const int wx = im.box[0], wy = im.box[1];
    const int vol = wx * wy * im.box[2];
    const double inv2h = 1.0 / (2.0 * c.h);
    for (int li = threadIdx.x; li < vol; li += CEN_THREADS) {
      const int sx = im.lo[0] + li % wx;
      const int sy = im.lo[1] + (li / wx) % wy;
      const int sz = im.lo[2] + li / (wx * wy);
      const long long n = node_index(g, sx, sy, sz);
      if (!c.an.band[n]) continue;
      const int2 et = c.an.tag[n];
      const int s = et.x == im.tag ? 0 : (et.y == im.tag ? 1 : -1);
      if (s < 0) continue;
      const int hx = sx + g.off[0], hy = sy + g.off[1], hz = sz + g.off[2];
      double de[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        double xp[3] = {im.xl[0], im.xl[1], im.xl[2]}, xm[3] = {im.xl[0], im.xl[1], im.xl[2]};
        xp[a] = xlp[a];
        xm[a] = xlm[a];
        const double ep = eps_exact(g.dim, hx, hy, hz, xp, im.r, c.h0);
        const double em = eps_exact(g.dim, hx, hy, hz, xm, im.r, c.h0);
        de[a] = (ep - em) * inv2h;
      }
      if (c.xdot) {
        c.an.edot[2 * n + s] =
            c.xdot[3 * i] * de[0] + c.xdot[3 * i + 1] * de[1] + c.xdot[3 * i + 2] * de[2];
      } else {
        const uint8_t flag = c.tab.flag[n];
        int2 id = make_int2(0, 0);
        double2 e = make_double2(0.0, 0.0);
        if (flag) {
          id = c.tab.ids[n];
          e = c.tab.eps[n];
        }
        SlotWeights w;
        slot_weights(e.x, e.y, id.x > 0, id.y > 0, c.weighting, c.tau, w);
        const double chain = c.an.sigma[2 * n] * w.dBde[0][s] + c.an.sigma[2 * n + 1] * w.dBde[1][s];
#pragma unroll
        for (int a = 0; a < 3; ++a) acc[a] += chain * de[a];
      }
    }
  }
  if (c.xdot) return;
  __shared__ double red[CEN_THREADS / 32][3];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double x = acc[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[wid][a] = x;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double x = 0.0;
    for (int w = 0; w < CEN_THREADS / 32; ++w) x += red[w][threadIdx.x];
    c.out[3 * i + threadIdx.x] = x;
  }
}

// total drag of one step along d, summed over the images in their order
__global__ void adj_drag_kernel(const double* fh, int n, double d0, double d1, double d2,
                                double* out) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += d0 * fh[3 * i] + d1 * fh[3 * i + 1] + d2 * fh[3 * i + 2];
  *out = s;
}

// sum of the per-block partials, fixed order
constexpr int SUM_THREADS = 256;
__global__ void __launch_bounds__(SUM_THREADS) adj_sum_kernel(const double* part,
                                                              long long nblocks, double* out) {
  __shared__ double red[SUM_THREADS][ADJ_PART];
  double acc[ADJ_PART] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (long long b = threadIdx.x; b < nblocks; b += SUM_THREADS)
#pragma unroll
    for (int k = 0; k < ADJ_PART; ++k) acc[k] += part[b * ADJ_PART + k];
#pragma unroll
  for (int k = 0; k < ADJ_PART; ++k) red[threadIdx.x][k] = acc[k];
  __syncthreads();
  for (int s = SUM_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
#pragma unroll
      for (int k = 0; k < ADJ_PART; ++k) red[threadIdx.x][k] += red[threadIdx.x + s][k];
    __syncthreads();
  }
  if (threadIdx.x < ADJ_PART) out[threadIdx.x] = red[0][threadIdx.x];
}

}  // namespace

long long adj_blocks(const Geom& g) {
  return (long long)((g.S[0] + ADJ_THREADS - 1) / ADJ_THREADS) * g.S[1] * g.S[2];
}

cudaError_t launch_adj_entries(const AdjSetup& s, cudaStream_t st) {
  const long long total = (long long)s.g.S[0] * s.g.S[1] * s.g.S[2];
  adj_entries_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t launch_adj_step(const AdjParams& p, int tangent, cudaStream_t st) {
  const unsigned grid = (unsigned)adj_blocks(p.g);
  if (p.g.dim == 2) {
    if (tangent)
      tan_step_kernel<D2Q9><<<grid, ADJ_THREADS, 0, st>>>(p);
    else
      adj_step_kernel<D2Q9><<<grid, ADJ_THREADS, 0, st>>>(p);
  } else {
    if (tangent)
      tan_step_kernel<D3Q19><<<grid, ADJ_THREADS, 0, st>>>(p);
    else
      adj_step_kernel<D3Q19><<<grid, ADJ_THREADS, 0, st>>>(p);
  }
  return cudaGetLastError();
}

cudaError_t launch_adj_centre(const AdjCentre& c, cudaStream_t st) {
  if (c.n <= 0) return cudaSuccess;
  adj_centre_kernel<<<c.n, CEN_THREADS, 0, st>>>(c);
  return cudaGetLastError();
}

cudaError_t launch_adj_drag(const double* fh, int n, double d0, double d1, double d2,
                            double* out, cudaStream_t st) {
  adj_drag_kernel<<<1, 1, 0, st>>>(fh, n, d0, d1, d2, out);
  return cudaGetLastError();
}

cudaError_t launch_adj_sum(const double* part, long long nblocks, double* out, cudaStream_t st) {
  adj_sum_kernel<<<1, SUM_THREADS, 0, st>>>(part, nblocks, out);
  return cudaGetLastError();
}

}  // namespace lbmpsm
