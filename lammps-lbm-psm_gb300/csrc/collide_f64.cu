// collide_f64.cu -- FP64 "plain" path: fused macro / BGK-PSM collision /
// A-A streaming kernel and the Zou-He face kernel, keeping the reference's
// operand order so that results match the reference CPU code bit for bit.
// Compiled with -fmad=false (no contraction of a*b+c).
//
// Reference: LBMPSMBGKDynamics::compute_macro_values
// (src/LBM_PSM_BGK_dynamics.cpp:48-77), collisionAndStream
// (src/LBM_PSM_BGK_dynamics.h:40-114), feq / F_iq
// (src/LBM_PSM_dynamics.h:43-116), add_Fhyd (src/LBM_PSM_lattice.cpp:355-363),
// macroCollideStream (src/LBM_PSM_BGK_dynamics.cpp:81-109), ZouHeBC
// (src/LBM_PSM_zou_he_BC.cpp:25-398).
#include "lbmpsm_internal.cuh"

namespace lbmpsm {

// signed sum of the non-zero components of e (each in {-1,0,1}) times v, in
// axis order; equal to the reference's ex*vx + ey*vy + ez*vz for these e.
template <int cx, int cy, int cz>
__device__ __forceinline__ double edot(double vx, double vy, double vz) {
  double s = 0.0;
  bool first = true;
  if (cx != 0) {
    s = cx > 0 ? vx : -vx;
    first = false;
  }
  if (cy != 0) {
    if (first) {
      s = cy > 0 ? vy : -vy;
      first = false;
    } else {
      s = cy > 0 ? s + vy : s - vy;
    }
  }
  if (cz != 0) {
    if (first) {
      s = cz > 0 ? vz : -vz;
      first = false;
    } else {
      s = cz > 0 ? s + vz : s - vz;
    }
  }
  return s;
}

template <class L, int q>
struct Dir {
  static constexpr int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
};

// Per-node state for the PSM branch.
struct PsmNode {
  bool has1, has2;
  double B1, B2, oneMinusBtot;
  double us1[3], us2[3];
  double half1, half2;  // 0.5*|us|^2*invCs2
  double F1[3], F2[3];
};

template <class L, int q>
__device__ __forceinline__ void collide_q(double& fq, double rho, double ux, double uy,
                                          double uz, double usq_half, const CollideParams& p,
                                          const BoxParams& bp, bool psm, PsmNode& sn) {
  constexpr int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
  const double w = L::w(q);
  const double fi = fq;
  // feq (src/LBM_PSM_dynamics.h:43-59)
  const double eu = (q == 0) ? 0.0 : edot<cx, cy, cz>(ux, uy, uz);
  const double fi_eq = rho * w * (1.0 + eu * p.invCs2 + eu * eu * 0.5 * p.invCs4 - usq_half);
  // Guo forcing (src/LBM_PSM_dynamics.h:102-116), scaled by (1 - omega/2)
  double Fq = 0.0;
  if (bp.has_force) {
    const double a = ((double)cx - ux) * bp.F[0] + ((double)cy - uy) * bp.F[1] +
                     ((double)cz - uz) * bp.F[2];
    const double eF = (q == 0) ? 0.0 : edot<cx, cy, cz>(bp.F[0], bp.F[1], bp.F[2]);
    Fq = bp.guo_pref * (w * (a * p.invCs2 + (eu * p.invCs4 * eF)));
  }
  if (!psm) {
    fq = fi + (fi_eq - fi) * bp.omega + Fq;
    return;
  }
  double sc1 = 0.0, sc2 = 0.0;
  if (sn.has1) {
    // feq(iq, rho, uSolid) array overload (src/LBM_PSM_dynamics.h:72-85)
    const double eus = (q == 0) ? 0.0 : edot<cx, cy, cz>(sn.us1[0], sn.us1[1], sn.us1[2]);
    const double f0s = rho * w * (1.0 + eus * p.invCs2 + 0.5 * eus * eus * p.invCs4 - sn.half1);
    sc1 = f0s - fi + bp.one_minus_omega * (fi - fi_eq);
  }
  if (sn.has2) {
    const double eus = (q == 0) ? 0.0 : edot<cx, cy, cz>(sn.us2[0], sn.us2[1], sn.us2[2]);
    const double f0s = rho * w * (1.0 + eus * p.invCs2 + 0.5 * eus * eus * p.invCs4 - sn.half2);
    sc2 = f0s - fi + bp.one_minus_omega * (fi - fi_eq);
  }
  fq = fi + sn.oneMinusBtot * (fi_eq - fi) * bp.omega + sn.B1 * sc1 + sn.B2 * sc2 + Fq;
  // node force on the particles (add_Fhyd): F += -B*Omega_s*e
  if (sn.has1) {
    const double t = -sn.B1 * sc1;
    if (cx) sn.F1[0] = cx > 0 ? sn.F1[0] + t : sn.F1[0] - t;
    if (cy) sn.F1[1] = cy > 0 ? sn.F1[1] + t : sn.F1[1] - t;
    if (cz) sn.F1[2] = cz > 0 ? sn.F1[2] + t : sn.F1[2] - t;
  }
  if (sn.has2) {
    const double t = -sn.B2 * sc2;
    if (cx) sn.F2[0] = cx > 0 ? sn.F2[0] + t : sn.F2[0] - t;
    if (cy) sn.F2[1] = cy > 0 ? sn.F2[1] + t : sn.F2[1] - t;
    if (cz) sn.F2[2] = cz > 0 ? sn.F2[2] + t : sn.F2[2] - t;
  }
}

template <class L, int q>
struct CollideUnroll {
  __device__ __forceinline__ static void run(double* f, double rho, double ux, double uy,
                                             double uz, double usq_half,
                                             const CollideParams& p, const BoxParams& bp, bool psm,
                                             PsmNode& sn) {
    collide_q<L, q>(f[q], rho, ux, uy, uz, usq_half, p, bp, psm, sn);
    CollideUnroll<L, q + 1>::run(f, rho, ux, uy, uz, usq_half, p, bp, psm, sn);
  }
};
template <class L>
struct CollideUnroll<L, L::Q> {
  __device__ __forceinline__ static void run(double*, double, double, double, double, double,
                                             const CollideParams&, const BoxParams&, bool,
                                             PsmNode&) {}
};

// One node of the FP64 collide + A-A stream step.
template <class L, bool ODD>
__device__ __forceinline__ void collide_f64_node(const CollideParams& p, int sx, int sy, int sz) {
  constexpr int Q = L::Q;
  const Geom& g = p.g;
  const long long n = node_index(g, sx, sy, sz);
  const Nbr nb = make_nbr(g, sx, sy, sz);
  const BoxParams bp = p.box[box_of_z(g, sz)];  // copied: read once, before any store
  double* F = static_cast<double*>(p.f);
  // in place unless a separate source is given (recomputation of stored states)
  const double* Fin = p.fsrc ? static_cast<const double*>(p.fsrc) : F;
  const long long Np = g.Np;

  double f[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    // incoming population q comes from the node at -e_q
    const bool ok = nbr_ok(nb, -cx, -cy, -cz);
    if (!ODD) {
      f[q] = ok ? Fin[q * Np + n] : L::w(q);
    } else {
      const int o = nbr_off(nb, -cx, -cy, -cz);
      f[q] = ok ? Fin[L::opp(q) * Np + n + o] : L::w(q);
    }
  }

  // macro values (src/LBM_PSM_BGK_dynamics.cpp:48-77)
  double rho = 0.0;
#pragma unroll
  for (int q = 0; q < Q; ++q) rho = rho + f[q];
  double jx = 0.0, jy = 0.0, jz = 0.0;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    if (cx) jx = cx > 0 ? jx + f[q] : jx - f[q];
    if (cy) jy = cy > 0 ? jy + f[q] : jy - f[q];
    if (cz) jz = cz > 0 ? jz + f[q] : jz - f[q];
  }
  jx = jx + bp.F[0] * 0.5;
  jy = jy + bp.F[1] * 0.5;
  jz = jz + bp.F[2] * 0.5;
  const double ux = jx / rho, uy = jy / rho, uz = jz / rho;
  if (p.store_macro) {
    p.rho_out[n] = rho;
    p.u_out[3 * n + 0] = ux;
    p.u_out[3 * n + 1] = uy;
    p.u_out[3 * n + 2] = uz;
  }
  const double usq_half = 0.5 * (ux * ux + uy * uy + uz * uz) * p.invCs2;

  PsmNode sn;
  const uint8_t flag = p.tab.flag[n];
  const bool psm = flag != 0;
  if (psm) {
    const int2 id = p.tab.ids[n];
    const double2 e = p.tab.eps[n];
    const double* us = p.tab.us + 6 * n;
    sn.has1 = id.x > 0;
    sn.has2 = id.y > 0;
    double B1 = sn.has1 ? e.x : 0.0;
    double B2 = sn.has2 ? e.y : 0.0;
    if (p.weighting == 1) {  // Noble-Torczynski weighting (opt-in)
      const double tm = bp.tau - 0.5;
      if (sn.has1) B1 = B1 * tm / ((1.0 - B1) + tm);
      if (sn.has2) B2 = B2 * tm / ((1.0 - B2) + tm);
    }
    double Btot = B1 + B2;
    if (Btot > 1.0) {
      B1 = B1 / Btot;
      B2 = B2 / Btot;
      Btot = 1.0;
    }
    sn.B1 = B1;
    sn.B2 = B2;
    sn.oneMinusBtot = 1.0 - Btot;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      sn.us1[c] = sn.has1 ? us[c] : 0.0;
      sn.us2[c] = sn.has2 ? us[3 + c] : 0.0;
      sn.F1[c] = 0.0;
      sn.F2[c] = 0.0;
    }
    sn.half1 = 0.5 * (sn.us1[0] * sn.us1[0] + sn.us1[1] * sn.us1[1] + sn.us1[2] * sn.us1[2]) * p.invCs2;
    sn.half2 = 0.5 * (sn.us2[0] * sn.us2[0] + sn.us2[1] * sn.us2[1] + sn.us2[2] * sn.us2[2]) * p.invCs2;
  } else {
    sn.has1 = sn.has2 = false;
    sn.B1 = sn.B2 = 0.0;
    sn.oneMinusBtot = 1.0;
    sn.half1 = sn.half2 = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      sn.us1[c] = sn.us2[c] = 0.0;
      sn.F1[c] = sn.F2[c] = 0.0;
    }
  }

  CollideUnroll<L, 0>::run(f, rho, ux, uy, uz, usq_half, p, bp, psm, sn);

  if (psm) {
    double* nf = static_cast<double*>(p.tab.nodeF) + 6 * n;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      nf[c] = sn.F1[c];
      nf[3 + c] = sn.F2[c];
    }
  }

#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
    if (!ODD) {
      F[L::opp(q) * Np + n] = f[q];
    } else {
      if (nbr_ok(nb, cx, cy, cz)) F[q * Np + n + nbr_off(nb, cx, cy, cz)] = f[q];
    }
  }
}

template <class L, bool ODD>
__global__ void __launch_bounds__(128) collide_f64_kernel(CollideParams p) {
  const Geom& g = p.g;
  // blocks: (row, x-chunk) folded into blockIdx.x (rows can exceed the 65535 limit of y)
  const int xblocks = (g.S[0] + blockDim.x - 1) / blockDim.x;
  const int row = blockIdx.x / xblocks;
  const int sx = (blockIdx.x - row * xblocks) * blockDim.x + threadIdx.x;
  if (sx >= g.S[0]) return;
  const int sy = row % g.S[1];
  const int sz = row / g.S[1];
  collide_f64_node<L, ODD>(p, sx, sy, sz);
}

// The members of a group in one launch: member m owns blocks
// [first[m], first[m+1]), laid out as its own kernel's (row, x-chunk) blocks;
// every node runs the same code as above, so the results are the members'.
template <class L, bool ODD>
__global__ void __launch_bounds__(128) collide_f64_multi_kernel(MultiCollide mc) {
  const int b = blockIdx.x;
  int m = 0;
  while (m + 1 < mc.nm && b >= mc.first[m + 1]) ++m;
  const CollideParams& p = mc.m[m].p;
  const Geom& g = p.g;
  const int S0 = g.S[0], S1 = g.S[1];
  const int xblocks = (S0 + blockDim.x - 1) / blockDim.x;
  const int lb = b - mc.first[m];
  const int row = lb / xblocks;
  const int sx = (lb - row * xblocks) * blockDim.x + threadIdx.x;
  if (sx >= S0) return;
  collide_f64_node<L, ODD>(p, sx, row % S1, row / S1);
}

cudaError_t launch_collide_f64_multi(const MultiCollide& mc, int odd, cudaStream_t st) {
  const unsigned grid = (unsigned)mc.first[mc.nm];
  if (grid == 0) return cudaSuccess;
  if (odd)
    collide_f64_multi_kernel<D3Q19, true><<<grid, 128, 0, st>>>(mc);
  else
    collide_f64_multi_kernel<D3Q19, false><<<grid, 128, 0, st>>>(mc);
  return cudaGetLastError();
}

template <class L>
static cudaError_t launch_collide_impl(const CollideParams& p, int odd, cudaStream_t st) {
  const Geom& g = p.g;
  dim3 block(128);
  dim3 grid((unsigned)(((g.S[0] + block.x - 1) / block.x) * (long long)g.S[1] * g.S[2]));
  if (odd)
    collide_f64_kernel<L, true><<<grid, block, 0, st>>>(p);
  else
    collide_f64_kernel<L, false><<<grid, block, 0, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_collide_f64(const CollideParams& p, int odd, cudaStream_t st) {
  return p.g.dim == 2 ? launch_collide_impl<D2Q9>(p, odd, st)
                      : launch_collide_impl<D3Q19>(p, odd, st);
}

// ------------------------------------------------------------------ Zou-He
// Exact restatements of the ZouHeBC members on one node's populations f[].
__device__ void zh_apply_f64(int kind, double* f, double p0) {
  const double o3 = 1.0 / 3.0, o6 = 1.0 / 6.0, t3 = 2.0 / 3.0;
  switch (kind) {
    case FACE_VEL2_XN: {  // :25-40
      const double ux = p0;
      double rho = 1.0 / (1.0 - ux) * (f[0] + f[2] + f[4] + 2.0 * (f[3] + f[6] + f[7]));
      f[5] = f[7] + 0.5 * (f[4] - f[2]) + rho * ux * o6;
      f[8] = f[6] + 0.5 * (f[2] - f[4]) + rho * ux * o6;
      f[1] = f[3] + t3 * rho * ux;
    } break;
    case FACE_VEL2_XP: {  // :43-58
      const double ux = p0;
      double rho = 1.0 / (1.0 - ux) * (f[0] + f[2] + f[4] + 2.0 * (f[1] + f[5] + f[8]));
      f[7] = f[5] + 0.5 * (f[2] - f[4]) - rho * ux * o6;
      f[6] = f[8] + 0.5 * (f[4] - f[2]) - rho * ux * o6;
      f[3] = f[1] - t3 * rho * ux;
    } break;
    case FACE_DENS2_XP: {  // :61-76
      const double rb = p0;
      double ux = -1.0 + 1.0 / rb * (f[0] + f[2] + f[4] + 2.0 * (f[1] + f[5] + f[8]));
      f[6] = f[8] + 0.5 * (f[4] - f[2]) - rb * ux * o6;
      f[7] = f[5] + 0.5 * (f[2] - f[4]) - rb * ux * o6;
      f[3] = f[1] - t3 * rb * ux;
    } break;
    case FACE_VEL2_YN: {  // :79-94
      const double ux = p0;
      double rho = f[0] + f[3] + f[1] + 2.0 * (f[8] + f[4] + f[7]);
      f[6] = f[8] + 0.5 * (f[1] - f[3]) - rho * ux * 0.5;
      f[5] = f[7] + 0.5 * (f[3] - f[1]) + rho * ux * 0.5;
      f[2] = f[4];
    } break;
    case FACE_VEL2_YP: {  // :97-112
      const double ux = p0;
      double rho = f[0] + f[3] + f[1] + 2.0 * (f[6] + f[2] + f[5]);
      f[7] = f[5] + 0.5 * (f[1] - f[3]) - rho * ux * 0.5;
      f[8] = f[6] + 0.5 * (f[3] - f[1]) + rho * ux * 0.5;
      f[4] = f[2];
    } break;
    case FACE_VEL3_XN: {  // :153-185 (uy = uz = 0 at every call site)
      const double ux = p0, uy = 0.0, uz = 0.0;
      double rho = 1.0 / (1.0 - ux) *
                   (f[0] + f[3] + f[4] + f[5] + f[6] + f[11] + f[17] + f[18] + f[12] +
                    2.0 * (f[2] + f[14] + f[8] + f[16] + f[10]));
      double Nyx = 0.5 * (f[3] + f[11] + f[17] - (f[4] + f[18] + f[12])) - o3 * rho * uy;
      double Nzx = 0.5 * (f[5] + f[18] + f[11] - (f[6] + f[17] + f[12])) - o3 * rho * uz;
      f[1] = f[2] + o3 * rho * ux;
      f[13] = f[14] + rho * o6 * (ux - uy) + Nyx;
      f[7] = f[8] + rho * o6 * (ux + uy) - Nyx;
      f[9] = f[10] + rho * o6 * (ux + uz) - Nzx;
      f[15] = f[16] + rho * o6 * (ux - uz) + Nzx;
    } break;
    case FACE_VEL3_XP: {  // :189-221
      const double ux = p0, uy = 0.0, uz = 0.0;
      double rho = 1.0 / (1.0 + ux) *
                   (f[0] + f[3] + f[4] + f[5] + f[6] + f[11] + f[17] + f[18] + f[12] +
                    2.0 * (f[1] + f[7] + f[13] + f[9] + f[15]));
      double Nyx = 0.5 * (f[3] + f[11] + f[17] - (f[4] + f[18] + f[12])) - o3 * rho * uy;
      double Nzx = 0.5 * (f[5] + f[18] + f[11] - (f[6] + f[17] + f[12])) - o3 * rho * uz;
      f[2] = f[1] - o3 * rho * ux;
      f[14] = f[13] + rho * o6 * (-ux + uy) - Nyx;
      f[8] = f[7] + rho * o6 * (-ux - uy) + Nyx;
      f[10] = f[9] + rho * o6 * (-ux - uz) + Nzx;
      f[16] = f[15] + rho * o6 * (-ux + uz) - Nzx;
    } break;
    case FACE_DENS3_XP: {  // :225-257
      const double rb = p0, uy = 0.0, uz = 0.0;
      double ux = -1.0 + 1.0 / rb *
                             (f[0] + f[3] + f[4] + f[5] + f[6] + f[11] + f[17] + f[18] + f[12] +
                              2.0 * (f[1] + f[7] + f[13] + f[9] + f[15]));
      double Nyx = 0.5 * (f[3] + f[11] + f[17] - (f[4] + f[18] + f[12])) - o3 * rb * uy;
      double Nzx = 0.5 * (f[5] + f[18] + f[11] - (f[6] + f[17] + f[12])) - o3 * rb * uz;
      f[2] = f[1] - o3 * rb * ux;
      f[14] = f[13] + rb * o6 * (-ux + uy) - Nyx;
      f[8] = f[7] + rb * o6 * (-ux - uy) + Nyx;
      f[10] = f[9] + rb * o6 * (-ux - uz) + Nzx;
      f[16] = f[15] + rb * o6 * (-ux + uz) - Nzx;
    } break;
    case FACE_VEL3_YN: {  // :261-293
      const double ux = p0, uy = 0.0, uz = 0.0;
      double rho = 1.0 / (1.0 - uy) *
                   (f[0] + f[1] + f[2] + f[5] + f[6] + f[9] + f[15] + f[16] + f[10] +
                    2.0 * (f[4] + f[13] + f[8] + f[18] + f[12]));
      double Nxy = 0.5 * (f[1] + f[9] + f[15] - (f[2] + f[16] + f[10])) - o3 * rho * ux;
      double Nzy = 0.5 * (f[5] + f[9] + f[16] - (f[6] + f[15] + f[10])) - o3 * rho * uz;
      f[3] = f[4] + o3 * rho * uy;
      f[7] = f[8] + rho * o6 * (uy + ux) - Nxy;
      f[14] = f[13] + rho * o6 * (uy - ux) + Nxy;
      f[11] = f[12] + rho * o6 * (uy + uz) - Nzy;
      f[17] = f[18] + rho * o6 * (uy - uz) + Nzy;
    } break;
    case FACE_VEL3_YP: {  // :296-328
      const double ux = p0, uy = 0.0, uz = 0.0;
      double rho = 1.0 / (1.0 + uy) *
                   (f[0] + f[1] + f[2] + f[5] + f[6] + f[9] + f[15] + f[16] + f[10] +
                    2.0 * (f[3] + f[7] + f[14] + f[11] + f[17]));
      double Nxy = 0.5 * (f[1] + f[9] + f[15] - (f[2] + f[16] + f[10])) - o3 * rho * ux;
      double Nzy = 0.5 * (f[5] + f[9] + f[16] - (f[6] + f[15] + f[10])) - o3 * rho * uz;
      f[4] = f[3] - o3 * rho * uy;
      f[8] = f[7] + rho * o6 * (-uy - ux) + Nxy;
      f[13] = f[14] + rho * o6 * (-uy + ux) - Nxy;
      f[12] = f[11] + rho * o6 * (-uy - uz) + Nzy;
      f[18] = f[17] + rho * o6 * (-uy + uz) - Nzy;
    } break;
    case FACE_VEL3_ZN: {  // :331-363
      const double ux = p0, uy = 0.0, uz = 0.0;
      double rho = 1.0 / (1.0 - uz) *
                   (f[0] + f[1] + f[2] + f[3] + f[4] + f[7] + f[13] + f[14] + f[8] +
                    2.0 * (f[6] + f[15] + f[10] + f[17] + f[12]));
      double Nxz = 0.5 * (f[1] + f[7] + f[13] - (f[2] + f[14] + f[8])) - o3 * rho * ux;
      double Nyz = 0.5 * (f[3] + f[7] + f[14] - (f[4] + f[13] + f[8])) - o3 * rho * uy;
      f[5] = f[6] + o3 * rho * uz;
      f[9] = f[10] + rho * o6 * (uz + ux) - Nxz;
      f[16] = f[15] + rho * o6 * (uz - ux) + Nxz;
      f[11] = f[12] + rho * o6 * (uz + uy) - Nyz;
      f[18] = f[17] + rho * o6 * (uz - uy) + Nyz;
    } break;
    case FACE_VEL3_ZP: {  // :366-398
      const double ux = p0, uy = 0.0, uz = 0.0;
      double rho = 1.0 / (1.0 + uz) *
                   (f[0] + f[1] + f[2] + f[3] + f[4] + f[7] + f[14] + f[8] + f[13] +
                    2.0 * (f[5] + f[9] + f[16] + f[11] + f[18]));
      double Nxz = 0.5 * (f[1] + f[7] + f[13] - (f[2] + f[14] + f[8])) - o3 * rho * ux;
      double Nyz = 0.5 * (f[3] + f[7] + f[14] - (f[4] + f[13] + f[8])) - o3 * rho * uy;
      f[6] = f[5] - o3 * rho * uz;
      f[15] = f[16] + rho * o6 * (-uz + ux) - Nxz;
      f[10] = f[9] + rho * o6 * (-uz - ux) + Nxz;
      f[17] = f[18] + rho * o6 * (-uz + uy) - Nyz;
      f[12] = f[11] + rho * o6 * (-uz - uy) + Nyz;
    } break;
    default:
      break;
  }
}

__device__ __forceinline__ bool face_contains(const Face& fc, int sx, int sy, int sz) {
  return sx >= fc.lo[0] && sx <= fc.hi[0] && sy >= fc.lo[1] && sy <= fc.hi[1] &&
         sz >= fc.lo[2] && sz <= fc.hi[2];
}

// Location of the post-stream population q of node n: after an even step it
// sits in the upstream node's opposite slot, after an odd step in the node's
// own slot.  Returns -1 when the upstream node does not exist (constant).
template <class L>
__device__ __forceinline__ long long post_stream_loc(const Geom& g, const Nbr& nb, long long n,
                                                     int q, int after_odd) {
  const int cx = L::ex(q), cy = L::ey(q), cz = L::ez(q);
  if (!nbr_ok(nb, -cx, -cy, -cz)) return -1;
  if (after_odd) return (long long)q * g.Np + n;
  return (long long)L::opp(q) * g.Np + n + nbr_off(nb, -cx, -cy, -cz);
}

// One thread per (face, node of the face); the node is processed by the
// first face of the list that contains it, which then applies every face
// containing the node in list order (the reference applies whole faces one
// after another, and each face call touches only the node's own populations).
template <class L>
__global__ void bc_f64_kernel(BCParams p) {
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
    if (face_contains(p.face[k], sx, sy, sz)) return;
  const Geom& g = p.g;
  const Nbr nb = make_nbr(g, sx, sy, sz);
  const long long n = node_index(g, sx, sy, sz);
  double* F = static_cast<double*>(p.f);
  double f[Q];
  long long loc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    loc[q] = post_stream_loc<L>(g, nb, n, q, p.after_odd);
    f[q] = loc[q] >= 0 ? F[loc[q]] : L::w(q);
  }
  for (int k = fi; k < p.nfaces; ++k)
    if (face_contains(p.face[k], sx, sy, sz)) zh_apply_f64(p.face[k].kind, f, p.face[k].p0);
#pragma unroll
  for (int q = 0; q < Q; ++q)
    if (loc[q] >= 0) F[loc[q]] = f[q];
}

cudaError_t launch_bc_f64(const BCParams& p, cudaStream_t st) {
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
    bc_f64_kernel<D2Q9><<<grid, block, 0, st>>>(p);
  else
    bc_f64_kernel<D3Q19><<<grid, block, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace lbmpsm
