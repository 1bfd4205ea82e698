// capi.cu -- the extern "C" boundary of liblbmpsm_gb300.so (include/lbmpsm.h).
//
// A handle owns one lattice resident in HBM plus the particle-image buffers,
// a CUDA stream and pinned staging buffers.  Host-pointer calls stage their
// arrays through pinned memory with one copy each way per coupling step;
// *_device calls take device arrays and stay asynchronous.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/lbmpsm.h"
#include "lbmpsm_internal.cuh"

using namespace lbmpsm;

struct lbmpsm_handle {
  lbmpsm_fix_params prm{};
  lbmpsm_options opt{};
  Geom g{};
  double origin[3]{};
  // UnitConversion (src/LBM_PSM_unitConversion.cpp:15-38)
  double nu_lb = 0, dx = 0, dx_d = 0, Uc = 0, u_lb = 0, dt_d = 0, tc = 0;
  double forceFactor = 0, torqueFactor = 0, volumeForceFactor = 0;
  double tau = 0, omega = 0, F_lbm[3]{};
  double invCs2 = 0, invCs4 = 0;
  bool has_force = false;
  int bc_type = 0;
  std::vector<Face> faces;
  long long t = 0;  // LBM steps done
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t aux = nullptr;                  // cell-list kernels of the map
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaEvent_t ev_bc_fork = nullptr, ev_bc_join = nullptr;  // the BC beside the reduction
  float scale16 = (float)(1 << FP16_SCALE_LOG2);
  // host-pointer steps without staging copies: the device reads and writes
  // pageable host memory through the host's page tables (NVLink-C2C on
  // Grace), so the image preparation reads the caller's image arrays and the
  // reduction writes the caller's outputs and status_host directly
  bool host_direct = false;
  int status_host = 0;
  // lattice
  void* f = nullptr;
  Table tab{};
  double* rho = nullptr;
  double* u = nullptr;
  bool macro_requested = false;
  bool macro_valid = false;
  // particles
  int cap = 0;
  long long list_cap = 0;
  int cb[3]{8, 8, 8}, C[3]{1, 1, 1};
  int* d_tag = nullptr;
  double* d_xvw = nullptr;  // x | v | omega | radius, each cap entries
  double* d_out = nullptr;  // fh | th | S  (12*cap)
  Img* d_img = nullptr;
  int4* d_arec = nullptr;   // compact image records of the table update (3 per image)
  int* d_cells = nullptr;   // count | off | fill (3*ncells)
  int* d_list = nullptr;
  int4* d_lrec = nullptr;  // records per cell-list entry (3 int4 each)
  unsigned short* d_sfcode = nullptr;  // solid-fraction codes of (image, box node) pairs
  long long sf_cap = 0;
  unsigned long long* d_pair_total = nullptr;  // [0] list pairs, [1] codes, [2] shell nodes
  int4* d_shell = nullptr;  // shell nodes of the solid-fraction map (sf_cap entries)
  int sm_count = 1;
  int* d_status = nullptr;
  double* d_check = nullptr;
  double* d_sf_value = nullptr;  // n/10^d for n = 0..1000
  float* d_sf_value32 = nullptr;  // its FP32 roundings
  void* h_stage = nullptr;  // pinned: inputs then outputs
  size_t h_stage_bytes = 0;
  int last_n = 0;
  // graphs of one step for each parity (map + collide + reduce + bc)
  cudaGraphExec_t gexec[2]{nullptr, nullptr};
  // graphs of one host-pointer step for each parity (upload of the staged
  // images, map + collide + reduce, download of the outputs and status word)
  cudaGraphExec_t hexec[2]{nullptr, nullptr};
  int hgraph_n = -1;
  int hprev_n = -1;   // image count of the previous host-pointer step
  int hsame = 0;      // consecutive host-pointer steps with that count
  PipeConfig pipe{};  // launch shape of the FP32/FP16 collide kernel
  long long full_wait_limit = 0;  // the collide pipeline consumers' wait limit (0: default)

  float tune_ms[LBMPSM_TUNE_CANDIDATES] = {-1.f, -1.f, -1.f, -1.f};
  bool tune_pending = false;  // the collide autotuner has yet to run
  int graph_n = -1;
  int graph_bc = -1;
  long long graph_gen = 0;  // bumped whenever captured graphs become stale (groups check it)
  size_t dev_bytes = 0;
  std::string err;
  // batched ensemble: nbox boxes stacked along z (one lattice: nbox = 1)
  int nbox = 1;
  std::vector<BoxParams> boxes;
  BoxParams* d_box = nullptr;
  int* d_img_box = nullptr;  // box of each image (cap entries)
  bool step_boxes = false;   // the current images carry box indices
  bool any_force = false;
  int sel_box = 0;           // box the reference-layout calls address
  double* out2[3]{};         // lbmpsm_step_device: the caller's F/T/S buffers, written by
                             // the reduction beside the handle's own (null otherwise)
  const void* src[5]{};      // the caller's tag, x, v, omega, radius arrays, read by the
                             // map in place and copied into d_tag / d_xvw (null otherwise)
  // graphs of one device-pointer step for each parity (map reading the
  // caller's images, collide, reduce); the image-preparation and reduce
  // nodes take each call's pointers
  cudaGraph_t dgraph[2]{nullptr, nullptr};
  cudaGraphExec_t dexec[2]{nullptr, nullptr};
  cudaGraphNode_t dprep[2]{nullptr, nullptr}, dreduce[2]{nullptr, nullptr};
  // the parameters those two nodes hold in the executable graph
  cudaKernelNodeParams dprep_kp[2]{}, dreduce_kp[2]{};
  MapParams dprep_p[2]{};
  ReduceParams dreduce_p[2]{};
  int dgraph_n = -1;
  int dprev_n = -1;  // image count of the previous device step
  int dsame = 0;     // consecutive device steps with that count
};

namespace {
thread_local std::string g_create_error;

int fail(lbmpsm_handle* h, int code, const std::string& msg) {
  if (h)
    h->err = msg;
  else
    g_create_error = msg;
  return code;
}

#define CUDA_TRY(h, call)                                                               \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail((h), e_ == cudaErrorMemoryAllocation ? LBMPSM_ERR_NOMEM : LBMPSM_ERR_CUDA, \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                  \
  } while (0)

template <typename T>
cudaError_t dmalloc(lbmpsm_handle* h, T** p, size_t bytes) {
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e == cudaSuccess) h->dev_bytes += bytes;
  return e;
}

void dfree(void* p) {
  if (p) cudaFree(p);
}

size_t storage_bytes(int storage) { return storage == 0 ? 8 : (storage == 1 ? 4 : 2); }  // FP16, BF16: 2

// Zou-He face calls of fix_LBM_PSM_BC::post_force (src/fix_LBM_PSM_BC.cpp:223-401)
// on one rank, converted from the reference halo frame to device storage.
void make_faces(lbmpsm_handle* h, int bc) {
  h->faces.clear();
  const Geom& g = h->g;
  const int ew = 1;
  const int nx = g.L[0], ny = g.L[1], nz = g.L[2];
  const double u = h->u_lb, rho_out = 1.0;
  auto add = [&](int kind, int axis, int plane, int a0, int a1, int b0, int b1, double p0) {
    Face fc{};
    fc.kind = kind;
    fc.axis = axis;
    int lo[3], hi[3];
    if (g.dim == 2) {
      if (axis == 0) {
        lo[0] = hi[0] = plane; lo[1] = a0; hi[1] = a1;
      } else {
        lo[1] = hi[1] = plane; lo[0] = a0; hi[0] = a1;
      }
      lo[2] = hi[2] = 0;
    } else {
      if (axis == 0) {
        lo[0] = hi[0] = plane; lo[1] = a0; hi[1] = a1; lo[2] = b0; hi[2] = b1;
      } else if (axis == 1) {
        lo[1] = hi[1] = plane; lo[0] = a0; hi[0] = a1; lo[2] = b0; hi[2] = b1;
      } else {
        lo[2] = hi[2] = plane; lo[0] = a0; hi[0] = a1; lo[1] = b0; hi[1] = b1;
      }
    }
    for (int d = 0; d < 3; ++d) {
      fc.lo[d] = lo[d] - g.off[d];
      fc.hi[d] = hi[d] - g.off[d];
      fc.lo[d] = std::max(fc.lo[d], 0);
      fc.hi[d] = std::min(fc.hi[d], g.S[d] - 1);
    }
    fc.plane = fc.lo[axis];
    fc.p0 = p0;
    if (fc.lo[0] <= fc.hi[0] && fc.lo[1] <= fc.hi[1] && fc.lo[2] <= fc.hi[2]) h->faces.push_back(fc);
  };
  if (g.dim == 2) {
    switch (bc) {
      case 1:
        add(FACE_VEL2_YN, 1, ew, ew, nx - 1 - ew, 0, 0, -u);
        add(FACE_VEL2_YP, 1, ny - 1 - ew, ew, nx - 1 - ew, 0, 0, u);
        break;
      case 2:
        add(FACE_VEL2_XN, 0, ew, ew, ny - 1 - ew, 0, 0, u);
        add(FACE_DENS2_XP, 0, nx - 1 - ew, ew, ny - 1 - ew, 0, 0, rho_out);
        add(FACE_VEL2_YN, 1, ew, 1 + ew, nx - 2 - ew, 0, 0, u);
        add(FACE_VEL2_YP, 1, ny - 1 - ew, 1 + ew, nx - 2 - ew, 0, 0, u);
        break;
      case 3:
        add(FACE_VEL2_YN, 1, ew, ew, nx - 1 - ew, 0, 0, 0.0);
        add(FACE_VEL2_YP, 1, ny - 1 - ew, ew, nx - 1 - ew, 0, 0, 0.0);
        break;
      case 4:
        add(FACE_VEL2_XN, 0, ew, ew, ny - 1 - ew, 0, 0, u);
        add(FACE_DENS2_XP, 0, nx - 1 - ew, ew, ny - 1 - ew, 0, 0, rho_out);
        add(FACE_VEL2_YN, 1, ew, ew, nx - 1 - ew, 0, 0, 0.0);
        add(FACE_VEL2_YP, 1, ny - 1 - ew, ew, nx - 1 - ew, 0, 0, 0.0);
        break;
      case 5:
        add(FACE_VEL2_XN, 0, ew, ew, ny - 1 - ew, 0, 0, 0.0);
        add(FACE_VEL2_XP, 0, nx - 1 - ew, ew, ny - 1 - ew, 0, 0, 0.0);
        add(FACE_VEL2_YN, 1, ew, ew, nx - 1 - ew, 0, 0, 0.0);
        add(FACE_VEL2_YP, 1, ny - 1 - ew, ew, nx - 1 - ew, 0, 0, 0.0);
        break;
      default:
        break;
    }
  } else {
    const int X0 = ew, X1 = nx - 1 - ew, Y0 = ew, Y1 = ny - 1 - ew, Z0 = ew, Z1 = nz - 1 - ew;
    switch (bc) {
      case 1:
        add(FACE_VEL3_YN, 1, ew, X0, X1, Z0, Z1, -u);
        add(FACE_VEL3_YP, 1, ny - 1 - ew, X0, X1, Z0, Z1, u);
        break;
      case 2:
        add(FACE_VEL3_XN, 0, ew, Y0, Y1, Z0, Z1, u);
        add(FACE_DENS3_XP, 0, nx - 1 - ew, Y0, Y1, Z0, Z1, rho_out);
        add(FACE_VEL3_YN, 1, ew, X0, X1, Z0, Z1, u);
        add(FACE_VEL3_YP, 1, ny - 1 - ew, X0, X1, Z0, Z1, u);
        add(FACE_VEL3_ZN, 2, ew, X0, X1, Y0, Y1, u);
        add(FACE_VEL3_ZP, 2, nz - 1 - ew, X0, X1, Y0, Y1, u);
        break;
      case 3:
        add(FACE_VEL3_YN, 1, ew, X0, X1, Z0, Z1, 0.0);
        add(FACE_VEL3_YP, 1, ny - 1 - ew, X0, X1, Z0, Z1, 0.0);
        break;
      case 4:
        add(FACE_VEL3_XN, 0, ew, Y0, Y1, Z0, Z1, u);
        add(FACE_DENS3_XP, 0, nx - 1 - ew, Y0, Y1, Z0, Z1, rho_out);
        add(FACE_VEL3_YN, 1, ew, X0, X1, Z0, Z1, 0.0);
        add(FACE_VEL3_YP, 1, ny - 1 - ew, X0, X1, Z0, Z1, 0.0);
        add(FACE_VEL3_ZN, 2, ew, X0, X1, Y0, Y1, 0.0);
        add(FACE_VEL3_ZP, 2, nz - 1 - ew, X0, X1, Y0, Y1, 0.0);
        break;
      case 5:
        add(FACE_VEL3_XN, 0, ew, Y0, Y1, Z0, Z1, 0.0);
        add(FACE_VEL3_XP, 0, nx - 1 - ew, Y0, Y1, Z0, Z1, 0.0);
        add(FACE_VEL3_YN, 1, ew, X0, X1, Z0, Z1, 0.0);
        add(FACE_VEL3_YP, 1, ny - 1 - ew, X0, X1, Z0, Z1, 0.0);
        add(FACE_VEL3_ZN, 2, ew, X0, X1, Y0, Y1, 0.0);
        add(FACE_VEL3_ZP, 2, nz - 1 - ew, X0, X1, Y0, Y1, 0.0);
        break;
      default:
        break;
    }
  }
}

void free_particles(lbmpsm_handle* h) {
  dfree(h->d_tag);
  dfree(h->d_xvw);
  dfree(h->d_out);
  dfree(h->d_img);
  dfree(h->d_arec);
  h->d_arec = nullptr;
  dfree(h->d_img_box);
  h->d_img_box = nullptr;
  dfree(h->d_list);
  dfree(h->d_lrec);
  h->d_lrec = nullptr;
  dfree(h->d_sfcode);
  dfree(h->d_shell);
  h->d_sfcode = nullptr;
  h->d_shell = nullptr;
  h->sf_cap = 0;
  h->d_tag = nullptr;
  h->d_xvw = nullptr;
  h->d_out = nullptr;
  h->d_img = nullptr;
  h->d_list = nullptr;
  if (h->h_stage) cudaFreeHost(h->h_stage);
  h->h_stage = nullptr;
  h->h_stage_bytes = 0;
}

void drop_run_graphs(lbmpsm_handle* h) {
  for (int k = 0; k < 2; ++k)
    if (h->gexec[k]) {
      cudaGraphExecDestroy(h->gexec[k]);
      h->gexec[k] = nullptr;
    }
  h->graph_n = -1;
}

void drop_host_graphs(lbmpsm_handle* h) {
  for (int k = 0; k < 2; ++k)
    if (h->hexec[k]) {
      cudaGraphExecDestroy(h->hexec[k]);
      h->hexec[k] = nullptr;
    }
  h->hgraph_n = -1;
}

void drop_device_graphs(lbmpsm_handle* h) {
  for (int k = 0; k < 2; ++k) {
    if (h->dexec[k]) cudaGraphExecDestroy(h->dexec[k]);
    if (h->dgraph[k]) cudaGraphDestroy(h->dgraph[k]);
    h->dexec[k] = nullptr;
    h->dgraph[k] = nullptr;
    h->dprep[k] = h->dreduce[k] = nullptr;
  }
  h->dgraph_n = -1;
}

void drop_graphs(lbmpsm_handle* h) {
  drop_run_graphs(h);
  drop_host_graphs(h);
  drop_device_graphs(h);
  h->graph_gen += 1;
}

// cells touched by one image box of width <= w nodes along each axis
long long cells_per_image(const lbmpsm_handle* h, double r_lb) {
  const double w = 2.0 * r_lb + 6.0;
  long long c = 1;
  for (int d = 0; d < 3; ++d) {
    long long nd = (long long)std::ceil(w / h->cb[d]) + 1;
    nd = std::min<long long>(nd, h->C[d]);
    c *= std::max<long long>(nd, 1);
  }
  return c;
}

int ensure_particles(lbmpsm_handle* h, int n, double max_r_phys) {
  if (n > h->cap) {
    drop_graphs(h);
    free_particles(h);
    int cap = std::max(n, std::max(h->cap * 2, 1024));
    CUDA_TRY(h, dmalloc(h, &h->d_tag, sizeof(int) * cap));
    CUDA_TRY(h, dmalloc(h, &h->d_xvw, sizeof(double) * 10 * cap));
    CUDA_TRY(h, dmalloc(h, &h->d_out, sizeof(double) * 12 * cap));
    CUDA_TRY(h, dmalloc(h, &h->d_img, sizeof(Img) * cap));
    CUDA_TRY(h, dmalloc(h, &h->d_arec, sizeof(int4) * 3 * cap));
    CUDA_TRY(h, dmalloc(h, &h->d_img_box, sizeof(int) * cap));
    h->h_stage_bytes = (2 * sizeof(int) + sizeof(double) * 10 + sizeof(double) * 12) * (size_t)cap + 64;
    CUDA_TRY(h, cudaMallocHost(&h->h_stage, h->h_stage_bytes));
    h->cap = cap;
    h->list_cap = 0;
  }
  // size the cell lists for the full image capacity, so that *_device calls
  // (which cannot grow buffers) never need more than was allocated
  const double r_lb = std::max(max_r_phys, h->opt.max_radius) / h->dx;
  const long long need = (long long)std::max(h->cap, 1) * cells_per_image(h, r_lb);
  if (need > h->list_cap) {
    drop_graphs(h);
    dfree(h->d_list);
    dfree(h->d_lrec);
    h->d_list = nullptr;
    h->d_lrec = nullptr;
    long long cap = std::max(need, 2 * h->list_cap);
    CUDA_TRY(h, dmalloc(h, &h->d_list, sizeof(int) * (size_t)cap));
    CUDA_TRY(h, dmalloc(h, &h->d_lrec, sizeof(int4) * 3 * (size_t)cap));
    h->list_cap = cap;
  }
  // solid-fraction codes: one per node of every image box, box edge <= 2r+6
  const double edge = std::ceil(2.0 * r_lb + 6.0);
  long long vol = 1;
  for (int d = 0; d < h->g.dim; ++d) vol *= (long long)std::min<double>(edge, h->g.S[d]);
  const long long need_sf = (long long)std::max(h->cap, 1) * vol;
  if (need_sf > h->sf_cap) {
    drop_graphs(h);
    dfree(h->d_sfcode);
    dfree(h->d_shell);
    h->d_sfcode = nullptr;
    h->d_shell = nullptr;
    long long cap = std::max(need_sf, 2 * h->sf_cap);
    CUDA_TRY(h, dmalloc(h, &h->d_sfcode, sizeof(unsigned short) * (size_t)cap));
    CUDA_TRY(h, dmalloc(h, &h->d_shell, sizeof(int4) * (size_t)cap));
    h->sf_cap = cap;
  }
  return LBMPSM_OK;
}

// The selected box of an ensemble seen as a lattice of its own: the same
// strides, one box's planes, every array offset to the box's first plane.
Geom box_geom(const lbmpsm_handle* h) {
  Geom g = h->g;
  g.S[2] = g.bz;
  g.nbox = 1;
  g.fbz = make_fastdiv((unsigned)g.bz);
  g.N = (long long)g.P0 * g.S[1] * g.bz;
  return g;
}
long long box_base(const lbmpsm_handle* h) {
  return (long long)h->sel_box * h->g.bz * h->g.S[1] * h->g.P0;
}
void* box_f(const lbmpsm_handle* h) {
  return static_cast<char*>(h->f) + box_base(h) * (long long)storage_bytes(h->opt.storage);
}
Table box_table(const lbmpsm_handle* h) {
  Table t = h->tab;
  const long long b = box_base(h);
  t.flag += b;
  t.ids += b;
  if (t.eps) t.eps += b;
  if (t.us) t.us += 6 * b;
  if (t.rec32) t.rec32 += 2 * b;
  t.nodeF = static_cast<char*>(t.nodeF) + 6 * b * (h->opt.storage == LBMPSM_STORAGE_FP64 ? 8 : 4);
  return t;
}

// the handle's collide parameters for its next step
CollideParams collide_params(const lbmpsm_handle* h) {
  CollideParams p{};
  p.g = h->g;
  p.f = h->f;
  p.tab = h->tab;
  p.store_macro = h->macro_requested ? 1 : 0;
  p.rho_out = h->rho;
  p.u_out = h->u;
  p.weighting = h->opt.psm_weighting;
  p.box = h->d_box;
  p.has_force = h->any_force ? 1 : 0;
  p.invCs2 = h->invCs2;
  p.invCs4 = h->invCs4;
  p.scale16 = h->scale16;
  p.status = h->d_status;
  p.pipe = h->pipe;
  p.full_wait_limit = h->full_wait_limit;
  return p;
}

// bookkeeping of a launched collide: the macro store is done, one step more
void collide_done(lbmpsm_handle* h) {
  if (h->macro_requested) {
    h->macro_requested = false;
    h->macro_valid = true;
  }
  h->t += 1;
}

int collide(lbmpsm_handle* h) {
  const CollideParams p = collide_params(h);
  const int odd = (int)(h->t & 1);
  cudaError_t e;
  switch (h->opt.storage) {
    case LBMPSM_STORAGE_FP64: e = launch_collide_f64(p, odd, h->stream); break;
    case LBMPSM_STORAGE_FP32: e = launch_collide_f32(p, odd, h->stream); break;
    case LBMPSM_STORAGE_BF16: e = launch_collide_bf16(p, odd, h->stream); break;
    default: e = launch_collide_f16(p, odd, h->stream); break;
  }
  CUDA_TRY(h, e);
  collide_done(h);
  return LBMPSM_OK;
}

// The collide autotuner (lbmpsm_options.collide_tuning): once the table
// holds the particles (from the second step on), every candidate launch shape
// runs a few even/odd step pairs on a scratch copy of the populations and the
// fastest is kept; the step graphs are rebuilt with it.  Skipped while the
// stream is being captured (it synchronises) and when the scratch copy cannot
// be allocated.  The trial collides write node forces, which the step's own
// collide rewrites for every node that holds a particle.
int maybe_tune(lbmpsm_handle* h) {
  if (!h->tune_pending || h->t < 1) return LBMPSM_OK;
  CUDA_TRY(h, cudaSetDevice(h->device));
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CUDA_TRY(h, cudaStreamIsCapturing(h->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return LBMPSM_OK;
  h->tune_pending = false;
  void* scratch = nullptr;
  const size_t bytes = storage_bytes(h->opt.storage) * (size_t)h->g.Np * h->g.Q;
  if (cudaMalloc(&scratch, bytes) != cudaSuccess) {
    cudaGetLastError();
    return LBMPSM_OK;
  }
  CollideParams p{};
  p.g = h->g;
  p.f = scratch;
  p.tab = h->tab;
  p.weighting = h->opt.psm_weighting;
  p.box = h->d_box;
  p.has_force = h->any_force ? 1 : 0;
  p.invCs2 = h->invCs2;
  p.invCs4 = h->invCs4;
  p.scale16 = h->scale16;
  p.status = h->d_status;
  PipeConfig best = h->pipe;
  cudaError_t e = cudaMemcpyAsync(scratch, h->f, bytes, cudaMemcpyDeviceToDevice, h->stream);
  if (e == cudaSuccess) e = tune_collide_lowp(p, h->opt.storage, h->sm_count, h->stream, &best, h->tune_ms);
  cudaStreamSynchronize(h->stream);
  cudaFree(scratch);
  CUDA_TRY(h, e);
  CUDA_TRY(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
  if (best.grid != h->pipe.grid || best.stages != h->pipe.stages) {
    h->pipe = best;
    drop_graphs(h);
  }
  return LBMPSM_OK;
}

// map -> collide -> reduce on device image arrays (internal buffers)
int enqueue_bc(lbmpsm_handle* h, cudaStream_t st);
// One coupling step (map, collide, reduce) on the handle's stream; with bc,
// also the boundary faces after the collide.  The faces touch only the
// populations, which neither the reduction nor the next step's map reads,
// so with images the face kernel runs on the auxiliary stream beside the
// reduction.
int enqueue_step(lbmpsm_handle* h, int n, bool bc = false);

// The particle map of a step with n images (nothing without images).
int enqueue_map(lbmpsm_handle* h, int n) {
  // image block layout: x | v | omega (3n each) | radius (n)
  const int* tag = h->d_tag;
  const double* x = h->d_xvw;
  const double* v = h->d_xvw + 3 * (size_t)n;
  const double* w = h->d_xvw + 6 * (size_t)n;
  const double* r = h->d_xvw + 9 * (size_t)n;
  if (n > 0) {
    const int ncells = h->C[0] * h->C[1] * h->C[2];
    CUDA_TRY(h, cudaMemsetAsync(h->d_cells, 0, sizeof(int) * 3 * (size_t)ncells, h->stream));
    CUDA_TRY(h, cudaMemsetAsync(h->d_pair_total, 0, 4 * sizeof(unsigned long long), h->stream));
    MapParams m{};
    m.g = h->g;
    m.tab = h->tab;
    m.n = n;
    m.tag = tag;
    m.x = x;
    m.v = v;
    m.omega = w;
    m.radius = r;
    if (h->src[0]) {  // read the caller's arrays; leave copies in the handle's buffers
      m.tag = static_cast<const int*>(h->src[0]);
      m.x = static_cast<const double*>(h->src[1]);
      m.v = static_cast<const double*>(h->src[2]);
      m.omega = static_cast<const double*>(h->src[3]);
      m.radius = static_cast<const double*>(h->src[4]);
      m.copy_tag = h->d_tag;
      m.copy_xvw = h->d_xvw;
    }
    m.img_box = h->step_boxes ? h->d_img_box : nullptr;
    m.box = h->d_box;
    m.dx = h->dx;
    m.sqrt2half = h->g.dim == 3 ? std::sqrt(3.1) / 2.0 : std::sqrt(2.1) / 2.0;
    m.img = h->d_img;
    m.arec = h->d_arec;
    for (int d = 0; d < 3; ++d) {
      m.cb[d] = h->cb[d];
      m.C[d] = h->C[d];
    }
    m.cell_count = h->d_cells;
    m.cell_off = h->d_cells + ncells;
    m.cell_fill = h->d_cells + 2 * (size_t)ncells;
    m.list = h->d_list;
    m.lrec = h->d_lrec;
    m.list_cap = h->list_cap;
    m.pair_total = h->d_pair_total;
    m.sfcode = h->d_sfcode;
    m.sf_cap = h->sf_cap;
    m.sf_value = h->d_sf_value;
    m.sf_value32 = h->d_sf_value32;
    m.shell = h->d_shell;
    m.shell_cap = h->sf_cap;
    m.sm_count = h->sm_count;
    m.status = h->d_status;
    m.write32 = h->opt.storage != LBMPSM_STORAGE_FP64 ? 1 : 0;
    CUDA_TRY(h, launch_map(m, h->stream, h->aux, h->ev_fork, h->ev_join));
  }
  return LBMPSM_OK;
}

// After the collide: the boundary faces (beside the reduction when there
// are images) and the reduction.
int enqueue_post(lbmpsm_handle* h, int n, bool bc) {
  const int* tag = h->d_tag;
  int rc = LBMPSM_OK;
  bool bc_aside = false;
  if (bc && !h->faces.empty()) {
    if (n > 0 && h->aux && h->ev_bc_fork && h->ev_bc_join) {
      CUDA_TRY(h, cudaEventRecord(h->ev_bc_fork, h->stream));
      CUDA_TRY(h, cudaStreamWaitEvent(h->aux, h->ev_bc_fork, 0));
      rc = enqueue_bc(h, h->aux);
      if (rc) return rc;
      CUDA_TRY(h, cudaEventRecord(h->ev_bc_join, h->aux));
      bc_aside = true;
    } else {
      rc = enqueue_bc(h, nullptr);
      if (rc) return rc;
    }
  }
  if (n > 0) {
    ReduceParams rp{};
    rp.img = h->d_img;
    rp.g = h->g;
    rp.tab = h->tab;
    rp.n = n;
    rp.tag = tag;
    rp.box = h->d_box;
    rp.nodeF_is_double = h->opt.storage == LBMPSM_STORAGE_FP64 ? 1 : 0;
    rp.fh = h->d_out;
    rp.th = h->d_out + 3 * (size_t)n;
    rp.S = h->d_out + 6 * (size_t)n;
    rp.fh2 = h->out2[0];
    rp.th2 = h->out2[1];
    rp.S2 = h->out2[2];
    rp.status = h->d_status;
    rp.status_out = h->host_direct ? &h->status_host : nullptr;
    CUDA_TRY(h, launch_reduce(rp, h->stream));
  }
  if (bc_aside) CUDA_TRY(h, cudaStreamWaitEvent(h->stream, h->ev_bc_join, 0));
  h->last_n = n;
  return LBMPSM_OK;
}

int enqueue_step(lbmpsm_handle* h, int n, bool bc) {
  int rc = enqueue_map(h, n);
  if (!rc) rc = collide(h);
  if (!rc) rc = enqueue_post(h, n, bc);
  return rc;
}

int enqueue_bc(lbmpsm_handle* h, cudaStream_t st) {
  if (h->faces.empty()) return LBMPSM_OK;
  if (!st) st = h->stream;
  BCParams b{};
  b.g = h->g;
  b.f = h->f;
  b.nfaces = (int)h->faces.size();
  for (int k = 0; k < b.nfaces; ++k) b.face[k] = h->faces[k];
  b.after_odd = (h->t % 2 == 0) ? 1 : 0;
  b.scale16 = h->scale16;
  cudaError_t e;
  switch (h->opt.storage) {
    case LBMPSM_STORAGE_FP64: e = launch_bc_f64(b, st); break;
    case LBMPSM_STORAGE_FP32: e = launch_bc_f32(b, st); break;
    case LBMPSM_STORAGE_BF16: e = launch_bc_bf16(b, st); break;
    default: e = launch_bc_f16(b, st); break;
  }
  CUDA_TRY(h, e);
  return LBMPSM_OK;
}

int read_status(lbmpsm_handle* h) {
  int st = 0;
  CUDA_TRY(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  if (st & STATUS_TIMEOUT) {
    CUDA_TRY(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
    return fail(h, LBMPSM_ERR_TIMEOUT, "a bounded device-side wait on a bulk copy gave up");
  }
  if (st & STATUS_LIST_OVERFLOW) {
    CUDA_TRY(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
    return fail(h, LBMPSM_ERR_CAPACITY,
                "particle cell lists overflowed: a radius exceeds the handle's max_radius");
  }
  return LBMPSM_OK;
}

bool finite_all(const double* a, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(a[i])) return false;
  return true;
}

}  // namespace

extern "C" {

const char* lbmpsm_last_error(const lbmpsm_handle* h) {
  return h ? h->err.c_str() : g_create_error.c_str();
}

}  // extern "C"

namespace {
// fix_LBM_PSM constructor and init checks (src/fix_LBM_PSM.cpp:15-83,122-140)
// and UnitConversion (src/LBM_PSM_unitConversion.cpp:15-38) of one box.
int box_setup(const lbmpsm_fix_params* p, BoxParams& bp, double& dx, double& volumeForceFactor,
              std::string& msg) {
  if (p->dimension != 2 && p->dimension != 3) {
    msg = "Illegal fix lbm-psm command: dimension must be 2 or 3";
    return LBMPSM_ERR_ARG;
  }
  if (p->nevery <= 0 || p->Nlc <= 0 || !(p->lc > 0.0) || !(p->rho > 0.0) || !(p->nu > 0.0) ||
      !(p->Re > 0.0) || !(p->tau > 0.5)) {
    msg = "Illegal fix lbm-psm command";
    return LBMPSM_ERR_ARG;
  }
  if (p->Nlc < 2) {
    msg = "Illegal fix lbm-psm command: Nlc must be > 1";
    return LBMPSM_ERR_ARG;
  }
  const double Uc_d = 1.0, Lc_d = 1.0, csPow2 = 1.0 / 3.0;
  const int N = p->Nlc;
  const double nu_lb = (p->tau - 0.5) * csPow2;
  dx = p->lc / (double)(N - 1);
  const double dx_d = Lc_d / (double)(N - 1);
  bp.Uc = p->Re * p->nu / p->lc;
  bp.u_lb = p->Re * nu_lb / (double)(N - 1);
  bp.dt_d = dx_d * bp.u_lb / Uc_d;
  bp.tc = p->lc / bp.Uc;
  bp.forceFactor = p->rho * pow(p->lc, 4) / pow(bp.tc, 2) * pow(dx_d, 4) / pow(bp.dt_d, 2);
  bp.torqueFactor = p->rho * pow(p->lc, 5) / pow(bp.tc, 2) * pow(dx_d, 5) / pow(bp.dt_d, 2);
  volumeForceFactor = p->rho * p->lc / pow(bp.tc, 2) * dx_d / pow(bp.dt_d, 2);
  const double Ma = bp.u_lb / (1.0 / sqrt(3.0));
  if (Ma > 0.3) {
    msg = "Mach number is Ma > 0.3. Aborting simulation. Choose parameters which give Ma < "
          "0.3 for stability reasons.";
    return LBMPSM_ERR_MACH;
  }
  const double SMALL = 1e-15;
  if (pow(((double)((int)(p->prd[0] / dx + 0.5)) - p->prd[0] / dx), 2.0) > SMALL ||
      pow(((double)((int)(p->prd[1] / dx + 0.5)) - p->prd[1] / dx), 2.0) > SMALL ||
      pow(((double)((int)(p->prd[2] / dx + 0.5)) - p->prd[2] / dx), 2.0) > SMALL) {
    msg = "Illegal cell width. Division of domain length and cell width has to give an "
          "integer.";
    return LBMPSM_ERR_GRID;
  }
  bp.origin[0] = p->boxlo[0];
  bp.origin[1] = p->boxlo[1];
  bp.origin[2] = p->dimension == 2 ? 0.0 : p->boxlo[2];
  for (int d = 0; d < 3; ++d) bp.F[d] = p->Fext[d] / volumeForceFactor;
  bp.has_force = (bp.F[0] * bp.F[0] + bp.F[1] * bp.F[1] + bp.F[2] * bp.F[2]) > 0.0 ? 1 : 0;
  bp.tau = p->tau;
  bp.omega = 1.0 / p->tau;
  bp.one_minus_omega = 1.0 - bp.omega;
  bp.guo_pref = (1.0 - 0.5 * bp.omega);
  // FP32 copies made on the host (double->float conversions are slow on the device)
  bp.omega_f = (float)bp.omega;
  bp.omo_f = (float)bp.one_minus_omega;
  bp.gpref_f = (float)bp.guo_pref;
  bp.tm_f = (float)(bp.tau - 0.5);
  for (int d = 0; d < 3; ++d) bp.F_f[d] = (float)bp.F[d];
  return LBMPSM_OK;
}

int create_impl(int nbox, const lbmpsm_fix_params* ps, const lbmpsm_options* opts,
                lbmpsm_handle** out) {
  if (!out) return fail(nullptr, LBMPSM_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (!ps) return fail(nullptr, LBMPSM_ERR_ARG, "params is NULL");
  if (nbox < 1) return fail(nullptr, LBMPSM_ERR_ARG, "an ensemble needs at least one box");
  const lbmpsm_fix_params* p = ps;
  lbmpsm_options o{};
  if (opts) o = *opts;
  if (o.storage < 0 || o.storage > 3)
    return fail(nullptr, LBMPSM_ERR_ARG, "unknown storage precision");
  if (o.psm_weighting < 0 || o.psm_weighting > 1)
    return fail(nullptr, LBMPSM_ERR_ARG, "unknown PSM weighting");
  std::vector<BoxParams> boxes((size_t)nbox);
  double dx = 0.0, vff = 0.0;
  for (int b = 0; b < nbox; ++b) {
    std::string msg;
    double dxb = 0.0, vffb = 0.0;
    const int rc = box_setup(&ps[b], boxes[(size_t)b], dxb, vffb, msg);
    if (rc) return fail(nullptr, rc, nbox > 1 ? "box " + std::to_string(b) + ": " + msg : msg);
    if (b == 0) {
      dx = dxb;
      vff = vffb;
      continue;
    }
    // one lattice geometry for every box of an ensemble
    const lbmpsm_fix_params& q = ps[b];
    bool same = q.dimension == p->dimension && dxb == dx;
    for (int d = 0; d < 3; ++d)
      same = same && q.prd[d] == p->prd[d] && (q.periodic[d] != 0) == (p->periodic[d] != 0);
    if (!same)
      return fail(nullptr, LBMPSM_ERR_ARG,
                  "box " + std::to_string(b) + ": the boxes of an ensemble must share dimension, "
                  "domain lengths, periodicity and lattice spacing");
  }

  lbmpsm_handle* h = new (std::nothrow) lbmpsm_handle();
  if (!h) return fail(nullptr, LBMPSM_ERR_NOMEM, "host allocation failed");
  h->prm = *p;
  h->opt = o;
  h->nbox = nbox;
  h->boxes = boxes;
  const BoxParams& b0 = boxes[0];
  h->dx = dx;
  h->dx_d = 1.0 / (double)(p->Nlc - 1);
  h->nu_lb = (p->tau - 0.5) / 3.0;
  h->Uc = b0.Uc;
  h->u_lb = b0.u_lb;
  h->dt_d = b0.dt_d;
  h->tc = b0.tc;
  h->forceFactor = b0.forceFactor;
  h->torqueFactor = b0.torqueFactor;
  h->volumeForceFactor = vff;
  int gn[3];
  gn[0] = p->prd[0] / dx + 1.5;
  if (p->periodic[0]) gn[0] -= 1;
  gn[1] = p->prd[1] / dx + 1.5;
  if (p->periodic[1]) gn[1] -= 1;
  gn[2] = 0;
  if (p->dimension == 3) {
    gn[2] = p->prd[2] / dx + 1.5;
    if (p->periodic[2]) gn[2] -= 1;
  }
  for (int d = 0; d < p->dimension; ++d)
    if (gn[d] < 1) {
      delete h;
      return fail(nullptr, LBMPSM_ERR_GRID, "lattice has no nodes along an axis");
    }
  for (int d = 0; d < 3; ++d) h->origin[d] = b0.origin[d];
  for (int d = 0; d < 3; ++d) h->F_lbm[d] = b0.F[d];
  h->has_force = b0.has_force != 0;
  h->any_force = false;
  for (const BoxParams& bp : boxes) h->any_force = h->any_force || bp.has_force;
  h->tau = p->tau;
  h->omega = 1.0 / p->tau;
  {
    const double csPow2 = 1.0 / 3.0, csPow4 = csPow2 * csPow2;
    h->invCs2 = 1.0 / csPow2;
    h->invCs4 = 1.0 / csPow4;
  }
  Geom& g = h->g;
  g.dim = p->dimension;
  g.Q = p->dimension == 2 ? 9 : 19;
  for (int d = 0; d < 3; ++d) {
    const bool real_axis = d < p->dimension;
    g.L[d] = real_axis ? gn[d] + 2 : 1;
    const bool per = !real_axis || p->periodic[d];
    g.per[d] = per ? 1 : 0;
    g.off[d] = (real_axis && per) ? 1 : 0;
    g.S[d] = (real_axis && per) ? gn[d] : g.L[d];
  }
  g.bz = g.S[2];
  g.nbox = nbox;
  g.fbz = make_fastdiv((unsigned)g.bz);
  g.S[2] = g.bz * nbox;
  if ((long long)g.S[2] > 65535 || g.L[0] > 65535 || g.L[1] > 65535) {
    delete h;
    return fail(nullptr, LBMPSM_ERR_GRID, "more than 65535 nodes along an axis");
  }
  g.P0 = (g.S[0] + 7) / 8 * 8;
  g.N = (long long)g.P0 * g.S[1] * g.S[2];
  g.Np = (g.N + 63) / 64 * 64;
  h->cb[0] = 8;
  h->cb[1] = 8;
  h->cb[2] = p->dimension == 3 ? 8 : 1;
  for (int d = 0; d < 3; ++d) h->C[d] = (g.S[d] + h->cb[d] - 1) / h->cb[d];

  h->device = o.device;
  auto bail = [&](int rc) {
    lbmpsm_destroy(h);
    return fail(nullptr, rc, "device set-up failed: " + std::string(cudaGetErrorString(cudaGetLastError())));
  };
  if (cudaSetDevice(h->device) != cudaSuccess) return bail(LBMPSM_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->aux, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_bc_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_bc_join, cudaEventDisableTiming) != cudaSuccess)
    return bail(LBMPSM_ERR_CUDA);
  const size_t es = storage_bytes(o.storage);
  const size_t N = (size_t)g.N;
  if (dmalloc(h, &h->f, es * (size_t)g.Np * g.Q) != cudaSuccess ||
      dmalloc(h, &h->tab.flag, N) != cudaSuccess ||
      dmalloc(h, &h->tab.ids, sizeof(int2) * N) != cudaSuccess ||
      dmalloc(h, &h->tab.nodeF, (o.storage == 0 ? 8 : 4) * 6 * N) != cudaSuccess)
    return bail(LBMPSM_ERR_NOMEM);
  // FP64 storage keeps the table in FP64; the other storages only the FP32 records
  if (o.storage == LBMPSM_STORAGE_FP64 &&
      (dmalloc(h, &h->tab.eps, sizeof(double2) * N) != cudaSuccess ||
       dmalloc(h, &h->tab.us, sizeof(double) * 6 * N) != cudaSuccess))
    return bail(LBMPSM_ERR_NOMEM);
  if (o.storage != LBMPSM_STORAGE_FP64 &&
      dmalloc(h, &h->tab.rec32, sizeof(float4) * 2 * N) != cudaSuccess)
    return bail(LBMPSM_ERR_NOMEM);
  const int ncells = h->C[0] * h->C[1] * h->C[2];
  if (dmalloc(h, &h->d_cells, sizeof(int) * 3 * (size_t)ncells) != cudaSuccess ||
      dmalloc(h, &h->d_pair_total, 4 * sizeof(unsigned long long)) != cudaSuccess ||
      dmalloc(h, &h->d_status, sizeof(int)) != cudaSuccess ||
      dmalloc(h, &h->d_check, sizeof(double) * (4 + 4 * 1024)) != cudaSuccess ||
      dmalloc(h, &h->d_sf_value, sizeof(double) * 1001) != cudaSuccess ||
      dmalloc(h, &h->d_sf_value32, sizeof(float) * 1001) != cudaSuccess)
    return bail(LBMPSM_ERR_NOMEM);
  {
    // calcSolidFraction's return value fraction*n (src/LBM_PSM_exchangeParticleData.cpp:165,213)
    double tbl[1001];
    const int slices = 10;
    double fraction = 1.0 / ((double)(slices * slices));
    if (g.dim == 3) fraction = 1.0 / ((double)(slices * slices * slices));
    for (int k = 0; k <= 1000; ++k) tbl[k] = fraction * ((double)k);
    float tbl32[1001];
    for (int k = 0; k <= 1000; ++k) tbl32[k] = (float)tbl[k];
    if (cudaMemcpy(h->d_sf_value, tbl, sizeof(tbl), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->d_sf_value32, tbl32, sizeof(tbl32), cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(LBMPSM_ERR_CUDA);
  }
  if (dmalloc(h, &h->d_box, sizeof(BoxParams) * (size_t)nbox) != cudaSuccess)
    return bail(LBMPSM_ERR_NOMEM);
  if (cudaMemcpy(h->d_box, h->boxes.data(), sizeof(BoxParams) * (size_t)nbox,
                 cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(LBMPSM_ERR_CUDA);
  cudaMemsetAsync(h->tab.flag, 0, N, h->stream);
  cudaMemsetAsync(h->tab.ids, 0, sizeof(int2) * N, h->stream);
  if (h->tab.eps) cudaMemsetAsync(h->tab.eps, 0, sizeof(double2) * N, h->stream);
  if (h->tab.us) cudaMemsetAsync(h->tab.us, 0, sizeof(double) * 6 * N, h->stream);
  cudaMemsetAsync(h->tab.nodeF, 0, (o.storage == 0 ? 8 : 4) * 6 * N, h->stream);
  if (h->tab.rec32) cudaMemsetAsync(h->tab.rec32, 0, sizeof(float4) * 2 * N, h->stream);
  cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream);
  if (launch_init_populations(g, h->f, o.storage, h->scale16, h->stream) != cudaSuccess)
    return bail(LBMPSM_ERR_CUDA);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, o.device) != cudaSuccess)
    return bail(LBMPSM_ERR_CUDA);
  h->sm_count = std::max(sms, 1);
  {
    int pageable = 0, host_tables = 0;
    const char* e = std::getenv("LBMPSM_HOST_STAGING");
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, o.device) == cudaSuccess &&
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                               o.device) == cudaSuccess)
      h->host_direct = pageable == 1 && host_tables == 1 && !(e && e[0] == '1');
    cudaGetLastError();
  }
  if (o.storage != LBMPSM_STORAGE_FP64) {
    // launch shape of the collide kernel: LBMPSM_PIPE_STAGES if set (0 = direct
    // kernel, 2..5 stages), else the autotuner or the 3-stage default
    const char* env = std::getenv("LBMPSM_PIPE_STAGES");
    const int stages = env ? std::atoi(env) : 3;
    if (prepare_collide_lowp(g, o.storage, sms, stages, &h->pipe) != cudaSuccess)
      return bail(LBMPSM_ERR_CUDA);
    // the autotuner runs at the start of the second step, when the first
    // step's map has filled the particle table
    h->tune_pending = !env && o.collide_tuning == LBMPSM_TUNE_AUTO;
    // test hook of the bounded-wait path: LBMPSM_TEST_FULL_WAIT_LIMIT=-1 makes
    // the pipeline's consumers give up on their first stage at once, so that a
    // step reports LBMPSM_ERR_TIMEOUT without any wait running long
    if (const char* wl = std::getenv("LBMPSM_TEST_FULL_WAIT_LIMIT"))
      h->full_wait_limit = std::atoll(wl);
  }
  int rc = ensure_particles(h, std::max(o.max_images, 1), o.max_radius > 0 ? o.max_radius : 8.0 * h->dx);
  if (rc) {
    std::string m = h->err;
    lbmpsm_destroy(h);
    return fail(nullptr, rc, m);
  }
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bail(LBMPSM_ERR_CUDA);
  *out = h;
  return LBMPSM_OK;
}
}  // namespace

extern "C" {

int lbmpsm_create(const lbmpsm_fix_params* p, const lbmpsm_options* opts, lbmpsm_handle** out) {
  return create_impl(1, p, opts, out);
}

int lbmpsm_create_batch(int nbox, const lbmpsm_fix_params* params, const lbmpsm_options* opts,
                        lbmpsm_handle** out) {
  return create_impl(nbox, params, opts, out);
}

void lbmpsm_destroy(lbmpsm_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graphs(h);
  free_particles(h);
  dfree(h->f);
  dfree(h->tab.flag);
  dfree(h->tab.ids);
  dfree(h->tab.eps);
  dfree(h->tab.us);
  dfree(h->tab.rec32);
  dfree(h->tab.nodeF);
  dfree(h->rho);
  dfree(h->u);
  dfree(h->d_cells);
  dfree(h->d_pair_total);
  dfree(h->d_status);
  dfree(h->d_check);
  dfree(h->d_sf_value);
  dfree(h->d_sf_value32);
  dfree(h->d_box);
  if (h->aux) cudaStreamSynchronize(h->aux);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->ev_bc_fork) cudaEventDestroy(h->ev_bc_fork);
  if (h->ev_bc_join) cudaEventDestroy(h->ev_bc_join);
  if (h->aux) cudaStreamDestroy(h->aux);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int lbmpsm_get_info(const lbmpsm_handle* h, lbmpsm_info* info) {
  if (!h || !info) return LBMPSM_ERR_ARG;
  info->dimension = h->g.dim;
  info->q = h->g.Q;
  info->nx = h->g.L[0] - 2;
  info->ny = h->g.L[1] - 2;
  info->nz = h->g.dim == 3 ? h->g.L[2] - 2 : 0;
  for (int d = 0; d < 3; ++d) {
    info->local[d] = h->g.L[d];
    info->storage_dims[d] = h->g.S[d];
  }
  info->dx = h->dx;
  info->Uc = h->Uc;
  info->u_lb = h->u_lb;
  info->tc = h->tc;
  info->dt_d = h->dt_d;
  info->forceFactor = h->forceFactor;
  info->torqueFactor = h->torqueFactor;
  info->volumeForceFactor = h->volumeForceFactor;
  info->dt_dem = (1.0 * h->dt_d * h->tc) / ((double)h->prm.nevery);
  info->Ma = h->u_lb / (1.0 / sqrt(3.0));
  for (int d = 0; d < 3; ++d) info->F_lbm[d] = h->F_lbm[d];
  info->steps = h->t;
  info->device_bytes = h->dev_bytes;
  info->collide_stages = h->opt.storage == LBMPSM_STORAGE_FP64 ? -1 : (h->pipe.grid > 0 ? h->pipe.stages : 0);
  info->collide_blocks = h->pipe.grid;
  for (int k = 0; k < LBMPSM_TUNE_CANDIDATES; ++k) info->collide_tune_ms[k] = h->tune_ms[k];
  return LBMPSM_OK;
}

int lbmpsm_select_box(lbmpsm_handle* h, int box) {
  if (!h) return LBMPSM_ERR_ARG;
  if (box < 0 || box >= h->nbox) return fail(h, LBMPSM_ERR_ARG, "box index out of range");
  h->sel_box = box;
  return LBMPSM_OK;
}

int lbmpsm_set_bc(lbmpsm_handle* h, int bc_type) {
  if (!h) return LBMPSM_ERR_ARG;
  if (h->nbox > 1 && bc_type != LBMPSM_BC_NONE)
    return fail(h, LBMPSM_ERR_STATE, "boundary conditions need a lattice of one box");
  if (bc_type < 0 || bc_type > 5) return fail(h, LBMPSM_ERR_ARG, "Illegal fix lbm-psm-bc command");
  h->bc_type = bc_type;
  make_faces(h, bc_type);
  drop_graphs(h);
  return LBMPSM_OK;
}

}  // extern "C"

namespace {
// pinned staging: tags | boxes | x | v | omega | radius (10*cap doubles from
// x on) | outputs (12*cap doubles) | status word
struct Stage {
  int* tag;
  int* box;
  double* xvw;
  double* out;
  int* status;
};
Stage stage_of(const lbmpsm_handle* h) {
  const size_t cap = (size_t)h->cap;
  char* st = static_cast<char*>(h->h_stage);
  const size_t iblk = (sizeof(int) * cap + 15) & ~(size_t)15;
  Stage s;
  s.tag = reinterpret_cast<int*>(st);
  s.box = reinterpret_cast<int*>(st + iblk);
  s.xvw = reinterpret_cast<double*>(st + 2 * iblk);
  s.out = s.xvw + 10 * cap;
  s.status = reinterpret_cast<int*>(s.out + 12 * cap);
  return s;
}

// copies of the staged images to the device buffers (enqueued on the stream)
int upload_images(lbmpsm_handle* h, int n) {
  if (n <= 0) return LBMPSM_OK;
  const Stage s = stage_of(h);
  const size_t nn = (size_t)n;
  CUDA_TRY(h, cudaMemcpyAsync(h->d_tag, s.tag, sizeof(int) * nn, cudaMemcpyHostToDevice, h->stream));
  if (h->step_boxes)
    CUDA_TRY(h, cudaMemcpyAsync(h->d_img_box, s.box, sizeof(int) * nn, cudaMemcpyHostToDevice,
                                h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(h->d_xvw, s.xvw, sizeof(double) * 10 * nn, cudaMemcpyHostToDevice,
                              h->stream));
  return LBMPSM_OK;
}

// Copy one set of particle images (host arrays) into pinned staging and,
// when upload is set, enqueue their copies to the handle's device buffers;
// box (may be null) gives each image's box.
int stage_images(lbmpsm_handle* h, int n, const int* box, const int* tag, const double* x,
                 const double* v, const double* omega, const double* radius, bool upload = true) {
  if (box) {
    for (int i = 0; i < n; ++i)
      if (box[i] < 0 || box[i] >= h->nbox)
        return fail(h, LBMPSM_ERR_ARG, "image " + std::to_string(i) + ": box index out of range");
  } else if (h->nbox > 1 && n > 0) {
    return fail(h, LBMPSM_ERR_ARG, "an ensemble needs the box of every image (lbmpsm_step_batch)");
  }
  CUDA_TRY(h, cudaSetDevice(h->device));
  double rmax = 0.0;
  for (int i = 0; i < n; ++i) rmax = std::max(rmax, radius[i]);
  if (!finite_all(x, 3 * (size_t)n) || !std::isfinite(rmax))
    return fail(h, LBMPSM_ERR_NUMERIC, "non-finite particle position or radius");
  int rc = ensure_particles(h, n, std::max(rmax, h->opt.max_radius));
  if (rc) return rc;
  const Stage sg = stage_of(h);
  int* stag = sg.tag;
  int* sbox = sg.box;
  double* sx = sg.xvw;
  if (h->step_boxes != (box != nullptr)) drop_graphs(h);  // the map reads the boxes or not
  h->step_boxes = box != nullptr;
  if (n > 0) {
    const size_t nn = (size_t)n;
    std::memcpy(stag, tag, sizeof(int) * nn);
    std::memcpy(sx, x, sizeof(double) * 3 * nn);
    std::memcpy(sx + 3 * nn, v, sizeof(double) * 3 * nn);
    std::memcpy(sx + 6 * nn, omega, sizeof(double) * 3 * nn);
    std::memcpy(sx + 9 * nn, radius, sizeof(double) * nn);
    if (box) std::memcpy(sbox, box, sizeof(int) * nn);
  }
  return upload ? upload_images(h, n) : LBMPSM_OK;
}

// One step from image arrays the device can read (device memory, or host
// memory when host_direct) into output arrays it can write: the map's image
// preparation reads the caller's arrays and copies them into the handle's
// buffers, the reduction writes the outputs beside the handle's own.
// Asynchronous on the handle's stream.
int device_step(lbmpsm_handle* h, int n, const int* tag, const double* x, const double* v,
                const double* omega, const double* radius, double* fh, double* th,
                double* stresslet) {
  auto enqueue_all = [&]() -> int {
    h->out2[0] = n > 0 ? fh : nullptr;
    h->out2[1] = n > 0 ? th : nullptr;
    h->out2[2] = n > 0 ? stresslet : nullptr;
    const void* src[5] = {tag, x, v, omega, radius};
    for (int k = 0; k < 5; ++k) h->src[k] = n > 0 ? src[k] : nullptr;
    const int r = enqueue_step(h, n);
    h->out2[0] = h->out2[1] = h->out2[2] = nullptr;
    for (int k = 0; k < 5; ++k) h->src[k] = nullptr;
    return r;
  };
  // Replayed as one CUDA graph per parity once the image count has held for
  // two calls (as host steps are); each call writes its own pointers into the
  // image-preparation and reduce nodes of the executable graph, which affects only the
  // launches that follow.  Steps that store the macroscopic fields, and steps
  // without images, run eagerly.
  h->dsame = n == h->dprev_n ? h->dsame + 1 : 0;
  h->dprev_n = n;
  if (n == 0 || h->macro_requested || (h->dgraph_n != n && h->dsame < 2)) return enqueue_all();
  if (h->dgraph_n != n) drop_device_graphs(h);
  const int par = (int)(h->t & 1);
  if (!h->dexec[par]) {
    cudaGraph_t graph = nullptr;
    CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const long long t0 = h->t;
    const int rc = enqueue_all();
    const cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    h->t = t0;  // captured, not run
    if (rc) {
      if (ce == cudaSuccess && graph) cudaGraphDestroy(graph);
      return rc;
    }
    CUDA_TRY(h, ce);
    // the nodes whose arguments change per call
    size_t nn = 0;
    cudaError_t e = cudaGraphGetNodes(graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (e == cudaSuccess) e = cudaGraphGetNodes(graph, nodes.data(), &nn);
    cudaGraphNode_t gn = nullptr, rn = nullptr;
    const void* fg = img_prep_fn();
    const void* fr = reduce_fn(h->opt.storage == LBMPSM_STORAGE_FP64 ? 1 : 0);
    for (size_t k = 0; e == cudaSuccess && k < nn; ++k) {
      cudaGraphNodeType ty;
      if (cudaGraphNodeGetType(nodes[k], &ty) != cudaSuccess || ty != cudaGraphNodeTypeKernel) continue;
      cudaKernelNodeParams kp{};
      if (cudaGraphKernelNodeGetParams(nodes[k], &kp) != cudaSuccess) continue;
      if (kp.func == fg) gn = nodes[k];
      if (kp.func == fr) rn = nodes[k];
    }
    cudaGraphExec_t ex = nullptr;
    if (e == cudaSuccess && gn && rn) e = cudaGraphInstantiate(&ex, graph, 0);
    if (e != cudaSuccess || !gn || !rn) {
      cudaGetLastError();
      cudaGraphDestroy(graph);
      CUDA_TRY(h, e);
      return fail(h, LBMPSM_ERR_CUDA,
                  "device-step graph: the image-preparation or reduce node was not found");
    }
    // the captured parameters (this call's pointers already)
    cudaKernelNodeParams kp{}, rk{};
    e = cudaGraphKernelNodeGetParams(gn, &kp);
    if (e == cudaSuccess) e = cudaGraphKernelNodeGetParams(rn, &rk);
    if (e != cudaSuccess) {
      cudaGraphExecDestroy(ex);
      cudaGraphDestroy(graph);
      CUDA_TRY(h, e);
    }
    h->dprep_p[par] = *static_cast<const MapParams*>(kp.kernelParams[0]);
    h->dreduce_p[par] = *static_cast<const ReduceParams*>(rk.kernelParams[0]);
    kp.kernelParams = nullptr;
    kp.extra = nullptr;
    rk.kernelParams = nullptr;
    rk.extra = nullptr;
    h->dprep_kp[par] = kp;
    h->dreduce_kp[par] = rk;
    h->dgraph[par] = graph;
    h->dexec[par] = ex;
    h->dprep[par] = gn;
    h->dreduce[par] = rn;
    h->dgraph_n = n;
  }
  {
    // this call's pointers into the image-preparation and reduce nodes, where
    // they differ from the ones the executable graph holds
    MapParams& mp = h->dprep_p[par];
    if (mp.tag != tag || mp.x != x || mp.v != v || mp.omega != omega || mp.radius != radius) {
      mp.tag = tag;
      mp.x = x;
      mp.v = v;
      mp.omega = omega;
      mp.radius = radius;
      void* ga[] = {(void*)&mp};
      cudaKernelNodeParams kp = h->dprep_kp[par];
      kp.kernelParams = ga;
      CUDA_TRY(h, cudaGraphExecKernelNodeSetParams(h->dexec[par], h->dprep[par], &kp));
    }
    ReduceParams& rp = h->dreduce_p[par];
    if (rp.fh2 != fh || rp.th2 != th || rp.S2 != stresslet) {
      rp.fh2 = fh;
      rp.th2 = th;
      rp.S2 = stresslet;
      void* ra[] = {(void*)&rp};
      cudaKernelNodeParams rk = h->dreduce_kp[par];
      rk.kernelParams = ra;
      CUDA_TRY(h, cudaGraphExecKernelNodeSetParams(h->dexec[par], h->dreduce[par], &rk));
    }
  }
  CUDA_TRY(h, cudaGraphLaunch(h->dexec[par], h->stream));
  h->t += 1;
  h->last_n = n;
  return LBMPSM_OK;
}

// one coupling step with host arrays; box (may be null) gives each image's box
//
// The device work of a step with images -- upload of the staged images, map,
// collide, reduce, download of the outputs and of the status word -- is
// captured once per A-A parity into a CUDA graph and replayed, so that a
// step costs one graph launch and one synchronisation on the host.  The
// graphs are keyed by the image count, which changes whenever a ghost image
// appears or goes: they are captured only once the count has held for two
// calls in a row, and steps before that run eagerly, as do steps that store
// the macroscopic fields.
int step_impl(lbmpsm_handle* h, int n, const int* box, const int* tag, const double* x,
              const double* v, const double* omega, const double* radius, double* fh, double* th,
              double* stresslet) {
  if (!h || n < 0) return LBMPSM_ERR_ARG;
  if (n > 0 && (!tag || !x || !v || !omega || !radius || !fh || !th || !stresslet))
    return fail(h, LBMPSM_ERR_ARG, "NULL particle array");
  int rc = maybe_tune(h);
  if (rc) return rc;
  if (h->host_direct && !box && h->nbox == 1 && n > 0) {
    // no staging: the device-step graph on the caller's host arrays
    CUDA_TRY(h, cudaSetDevice(h->device));
    double rmax = 0.0;
    for (int i = 0; i < n; ++i) rmax = std::max(rmax, radius[i]);
    if (!finite_all(x, 3 * (size_t)n) || !std::isfinite(rmax))
      return fail(h, LBMPSM_ERR_NUMERIC, "non-finite particle position or radius");
    rc = ensure_particles(h, n, std::max(rmax, h->opt.max_radius));
    if (rc) return rc;
    if (h->step_boxes) drop_graphs(h);
    h->step_boxes = false;
    h->status_host = 0;
    rc = device_step(h, n, tag, x, v, omega, radius, fh, th, stresslet);
    if (rc) return rc;
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return h->status_host ? read_status(h) : LBMPSM_OK;
  }
  rc = stage_images(h, n, box, tag, x, v, omega, radius, /*upload=*/false);
  if (rc) return rc;
  const Stage sg = stage_of(h);
  if (n == 0) {
    rc = enqueue_step(h, n);
    if (rc) return rc;
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return LBMPSM_OK;
  }
  const size_t nn = (size_t)n;
  auto enqueue_all = [&]() -> int {
    int r = upload_images(h, n);
    if (!r) r = enqueue_step(h, n);
    if (r) return r;
    CUDA_TRY(h, cudaMemcpyAsync(sg.out, h->d_out, sizeof(double) * 12 * nn,
                                cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(sg.status, h->d_status, sizeof(int), cudaMemcpyDeviceToHost,
                                h->stream));
    return LBMPSM_OK;
  };
  h->hsame = n == h->hprev_n ? h->hsame + 1 : 0;
  h->hprev_n = n;
  if (h->macro_requested || (h->hgraph_n != n && h->hsame < 2)) {
    rc = enqueue_all();
    if (rc) return rc;
  } else {
    if (h->hgraph_n != n) drop_host_graphs(h);
    const int par = (int)(h->t & 1);
    if (!h->hexec[par]) {
      cudaGraph_t graph = nullptr;
      CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      const long long t0 = h->t;
      rc = enqueue_all();
      cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
      h->t = t0;  // captured, not run
      if (rc) {
        if (ce == cudaSuccess && graph) cudaGraphDestroy(graph);
        return rc;
      }
      CUDA_TRY(h, ce);
      cudaError_t ie = cudaGraphInstantiate(&h->hexec[par], graph, 0);
      cudaGraphDestroy(graph);
      CUDA_TRY(h, ie);
      h->hgraph_n = n;
    }
    CUDA_TRY(h, cudaGraphLaunch(h->hexec[par], h->stream));
    h->t += 1;
    h->last_n = n;
  }
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  if (*sg.status) {
    rc = read_status(h);  // resets the device word and reports the error
    if (rc) return rc;
  }
  std::memcpy(fh, sg.out, sizeof(double) * 3 * nn);
  std::memcpy(th, sg.out + 3 * nn, sizeof(double) * 3 * nn);
  std::memcpy(stresslet, sg.out + 6 * nn, sizeof(double) * 6 * nn);
  return LBMPSM_OK;
}
}  // namespace

extern "C" {

int lbmpsm_step(lbmpsm_handle* h, int n, const int* tag, const double* x, const double* v,
                const double* omega, const double* radius, double* fh, double* th,
                double* stresslet) {
  return step_impl(h, n, nullptr, tag, x, v, omega, radius, fh, th, stresslet);
}

int lbmpsm_step_batch(lbmpsm_handle* h, int n, const int* box, const int* tag, const double* x,
                      const double* v, const double* omega, const double* radius, double* fh,
                      double* th, double* stresslet) {
  if (n > 0 && !box) return fail(h, LBMPSM_ERR_ARG, "NULL box array");
  return step_impl(h, n, box, tag, x, v, omega, radius, fh, th, stresslet);
}

int lbmpsm_step_device(lbmpsm_handle* h, int n, const int* tag, const double* x, const double* v,
                       const double* omega, const double* radius, double* fh, double* th,
                       double* stresslet) {
  if (!h || n < 0) return LBMPSM_ERR_ARG;
  if (n > h->cap) return fail(h, LBMPSM_ERR_CAPACITY, "more images than options.max_images");
  if (h->opt.max_radius <= 0.0)
    return fail(h, LBMPSM_ERR_ARG, "lbmpsm_step_device needs options.max_radius");
  if (h->nbox > 1 && n > 0)
    return fail(h, LBMPSM_ERR_ARG, "an ensemble needs the box of every image (lbmpsm_step_batch)");
  CUDA_TRY(h, cudaSetDevice(h->device));
  {
    const int trc = maybe_tune(h);
    if (trc) return trc;
  }
  if (h->step_boxes) drop_graphs(h);
  h->step_boxes = false;
  if (n > 0 && (!tag || !x || !v || !omega || !radius))
    return fail(h, LBMPSM_ERR_ARG, "NULL particle array");
  return device_step(h, n, tag, x, v, omega, radius, fh, th, stresslet);
}

int lbmpsm_apply_bc(lbmpsm_handle* h) {
  if (!h) return LBMPSM_ERR_ARG;
  CUDA_TRY(h, cudaSetDevice(h->device));
  return enqueue_bc(h, nullptr);
}

int lbmpsm_request_macro(lbmpsm_handle* h) {
  if (!h) return LBMPSM_ERR_ARG;
  if (!h->rho) {
    CUDA_TRY(h, cudaSetDevice(h->device));
    CUDA_TRY(h, dmalloc(h, &h->rho, sizeof(double) * (size_t)h->g.N));
    CUDA_TRY(h, dmalloc(h, &h->u, sizeof(double) * 3 * (size_t)h->g.N));
    drop_graphs(h);
  }
  h->macro_requested = true;
  return LBMPSM_OK;
}

int lbmpsm_export_fields(lbmpsm_handle* h, int as_double, double B0, double rho0, double u0,
                         void* solid, void* rho, void* u) {
  if (!h) return LBMPSM_ERR_ARG;
  CUDA_TRY(h, cudaSetDevice(h->device));
  const Geom g = box_geom(h);
  const long long base = box_base(h);
  const size_t npts = (size_t)(g.L[0] - 2) * (g.L[1] - 2) * (g.dim == 3 ? g.L[2] - 2 : 1);
  const size_t es = as_double ? 8 : 4;
  void* d = nullptr;
  CUDA_TRY(h, cudaMalloc(&d, es * 5 * npts));
  char* b = static_cast<char*>(d);
  cudaError_t e = launch_export_fields(g, box_table(h), h->macro_valid ? h->rho + base : nullptr,
                                       h->macro_valid ? h->u + 3 * base : nullptr, as_double, B0,
                                       rho0, u0, b, b + es * npts, b + 2 * es * npts, h->stream);
  if (e == cudaSuccess && solid) e = cudaMemcpyAsync(solid, b, es * npts, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && rho) e = cudaMemcpyAsync(rho, b + es * npts, es * npts, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && u) e = cudaMemcpyAsync(u, b + 2 * es * npts, 3 * es * npts, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  CUDA_TRY(h, e);
  return LBMPSM_OK;
}

int lbmpsm_get_populations(lbmpsm_handle* h, double* f) {
  if (!h || !f) return LBMPSM_ERR_ARG;
  CUDA_TRY(h, cudaSetDevice(h->device));
  const Geom g = box_geom(h);
  const size_t cnt = (size_t)g.L[0] * g.L[1] * g.L[2] * g.Q;
  double* d = nullptr;
  CUDA_TRY(h, cudaMalloc(&d, sizeof(double) * cnt));
  cudaError_t e = launch_get_populations(g, box_f(h), h->opt.storage, (h->t % 2 == 0) ? 1 : 0,
                                         h->scale16, d, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(f, d, sizeof(double) * cnt, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  CUDA_TRY(h, e);
  return LBMPSM_OK;
}

int lbmpsm_set_populations(lbmpsm_handle* h, const double* f) {
  if (!h || !f) return LBMPSM_ERR_ARG;
  CUDA_TRY(h, cudaSetDevice(h->device));
  const Geom g = box_geom(h);
  const size_t cnt = (size_t)g.L[0] * g.L[1] * g.L[2] * g.Q;
  double* d = nullptr;
  CUDA_TRY(h, cudaMalloc(&d, sizeof(double) * cnt));
  cudaError_t e = cudaMemcpyAsync(d, f, sizeof(double) * cnt, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess)
    e = launch_set_populations(g, box_f(h), h->opt.storage, (h->t % 2 == 0) ? 1 : 0, h->scale16,
                               d, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  CUDA_TRY(h, e);
  return LBMPSM_OK;
}

int lbmpsm_get_particle_table(lbmpsm_handle* h, int* ids, double* eps, double* us) {
  if (!h) return LBMPSM_ERR_ARG;
  CUDA_TRY(h, cudaSetDevice(h->device));
  const Geom g = box_geom(h);
  const size_t N = (size_t)g.L[0] * g.L[1] * g.L[2];
  void* d = nullptr;
  CUDA_TRY(h, cudaMalloc(&d, N * (2 * sizeof(int) + 8 * sizeof(double))));
  int* di = static_cast<int*>(d);
  double* de = reinterpret_cast<double*>(di + 2 * N);
  double* du = de + 2 * N;
  cudaError_t e = launch_table_export(g, box_table(h), di, de, du, h->stream);
  if (e == cudaSuccess && ids) e = cudaMemcpyAsync(ids, di, sizeof(int) * 2 * N, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && eps) e = cudaMemcpyAsync(eps, de, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && us) e = cudaMemcpyAsync(us, du, sizeof(double) * 6 * N, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  CUDA_TRY(h, e);
  return LBMPSM_OK;
}

int lbmpsm_check(lbmpsm_handle* h, double* mass, double* momentum3) {
  if (!h) return LBMPSM_ERR_ARG;
  CUDA_TRY(h, cudaSetDevice(h->device));
  CUDA_TRY(h, launch_check(h->g, h->f, h->opt.storage, (h->t % 2 == 0) ? 1 : 0, h->scale16,
                           h->d_check, h->d_status, h->stream));
  double acc[4];
  int st = 0;
  CUDA_TRY(h, cudaMemcpyAsync(acc, h->d_check, sizeof(acc), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  if (mass) *mass = acc[0];
  if (momentum3)
    for (int d = 0; d < 3; ++d) momentum3[d] = acc[1 + d];
  if (st & STATUS_NONFINITE) {
    CUDA_TRY(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
    return fail(h, LBMPSM_ERR_NUMERIC, "non-finite populations detected");
  }
  return LBMPSM_OK;
}

int lbmpsm_synchronize(lbmpsm_handle* h) {
  if (!h) return LBMPSM_ERR_ARG;
  CUDA_TRY(h, cudaSetDevice(h->device));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return read_status(h);
}

void* lbmpsm_stream(lbmpsm_handle* h) { return h ? (void*)h->stream : nullptr; }

int lbmpsm_host_direct(const lbmpsm_handle* h) { return h ? (h->host_direct ? 1 : 0) : -1; }

int lbmpsm_run_fixed(lbmpsm_handle* h, int nsteps) {
  if (!h || nsteps < 0) return LBMPSM_ERR_ARG;
  CUDA_TRY(h, cudaSetDevice(h->device));
  {
    const int trc = maybe_tune(h);
    if (trc) return trc;
  }
  const int n = h->last_n;
  const int use_bc = h->faces.empty() ? 0 : 1;
  if (h->graph_n != n || h->graph_bc != use_bc || h->macro_requested) drop_run_graphs(h);
  // a requested macro store runs eagerly (it changes the kernel arguments)
  while (nsteps > 0 && h->macro_requested) {
    int rc = enqueue_step(h, n, use_bc);
    if (rc) return rc;
    --nsteps;
  }
  for (int s = 0; s < nsteps; ++s) {
    const int par = (int)(h->t & 1);
    if (!h->gexec[par]) {
      cudaGraph_t graph = nullptr;
      CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      const long long t0 = h->t;
      int rc = enqueue_step(h, n, use_bc);
      cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
      h->t = t0;  // captured, not run
      if (rc) {
        if (ce == cudaSuccess && graph) cudaGraphDestroy(graph);
        return rc;
      }
      CUDA_TRY(h, ce);
      cudaError_t ie = cudaGraphInstantiate(&h->gexec[par], graph, 0);
      cudaGraphDestroy(graph);
      CUDA_TRY(h, ie);
      h->graph_n = n;
      h->graph_bc = use_bc;
    }
    CUDA_TRY(h, cudaGraphLaunch(h->gexec[par], h->stream));
    h->t += 1;
  }
  return LBMPSM_OK;
}

int lbmpsm_read_forces(lbmpsm_handle* h, int n, double* fh, double* th, double* stresslet) {
  if (!h || n < 0 || n > h->last_n) return LBMPSM_ERR_ARG;
  CUDA_TRY(h, cudaSetDevice(h->device));
  const size_t m = (size_t)h->last_n;
  if (fh) CUDA_TRY(h, cudaMemcpyAsync(fh, h->d_out, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->stream));
  if (th) CUDA_TRY(h, cudaMemcpyAsync(th, h->d_out + 3 * m, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->stream));
  if (stresslet) CUDA_TRY(h, cudaMemcpyAsync(stresslet, h->d_out + 6 * m, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return read_status(h);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free field export (lbmpsm_export_fields_static).
//
// lbmpsm_export_fields stages the fields through a device buffer that it
// cudaMalloc's and cudaFree's on every call.  Two kinds of caller cannot
// allow that in the middle of a run: a host program whose own pool allocator
// already holds nearly all of HBM, so that the cudaMalloc fails, and one that
// runs other streams on the same GPU, which cudaFree would stall because it
// waits for the whole device.  This variant stages through the fixed array
// below: LBMPSM_EXPORT_STATIC_MAX_BYTES (64 MiB) that every GPU loading the
// library holds until the process exits.  It launches the same export kernel
// as lbmpsm_export_fields and allocates nothing.
//
// In host code g_export_scratch only stands for the device array; its device
// address is looked up with cudaGetSymbolAddress once per device, with that
// device current, on the first call made for a handle on that device.  Make
// that first call before any stream capture begins.
//
// Every call on a device uses the same array and leaves its contents there.
// Nothing in it has to start at zero: the kernel writes every element that
// the copies then read back, so a previous call's data never reaches the
// caller.  Exports whose GPU work overlapped would race on the array; this
// function therefore holds a process-wide lock from its launch until its
// copies have finished, so its own calls run one after another.
static __device__ __align__(256) unsigned char g_export_scratch[LBMPSM_EXPORT_STATIC_MAX_BYTES];

namespace {
constexpr int kExportMaxDevices = 64;
std::mutex g_export_mutex;
void* g_export_addr[kExportMaxDevices] = {};  // device address of g_export_scratch
}  // namespace

extern "C" int lbmpsm_export_fields_static(lbmpsm_handle* h, int as_double, double B0,
                                           double rho0, double u0, void* solid, void* rho,
                                           void* u) {
  if (!h) return LBMPSM_ERR_ARG;
  if (h->device < 0 || h->device >= kExportMaxDevices)
    return fail(h, LBMPSM_ERR_ARG, "lbmpsm_export_fields_static: device index out of range");
  // the selected box of an ensemble, exactly as lbmpsm_export_fields addresses it
  const Geom g = box_geom(h);
  const long long base = box_base(h);
  const size_t npts = (size_t)(g.L[0] - 2) * (g.L[1] - 2) * (g.dim == 3 ? g.L[2] - 2 : 1);
  const size_t es = as_double ? 8 : 4;
  // only the requested fields are staged, packed solid | rho | u
  const size_t b_solid = solid ? es * npts : 0, b_rho = rho ? es * npts : 0,
               b_u = u ? 3 * es * npts : 0;
  const size_t need = b_solid + b_rho + b_u;
  if (need > (size_t)LBMPSM_EXPORT_STATIC_MAX_BYTES)
    return fail(h, LBMPSM_ERR_CAPACITY,
                "lbmpsm_export_fields_static: the requested fields of " + std::to_string(npts) +
                    " nodes need " + std::to_string(need) +
                    " bytes of scratch, more than its fixed " +
                    std::to_string((size_t)LBMPSM_EXPORT_STATIC_MAX_BYTES) +
                    "; request fewer fields, float output, or use lbmpsm_export_fields");
  if (need == 0) return LBMPSM_OK;
  CUDA_TRY(h, cudaSetDevice(h->device));
  std::lock_guard<std::mutex> lock(g_export_mutex);
  if (!g_export_addr[h->device]) {
    void* a = nullptr;
    CUDA_TRY(h, cudaGetSymbolAddress(&a, g_export_scratch));
    g_export_addr[h->device] = a;
  }
  char* b = static_cast<char*>(g_export_addr[h->device]);
  char* d_solid = solid ? b : nullptr;
  char* d_rho = rho ? b + b_solid : nullptr;
  char* d_u = u ? b + b_solid + b_rho : nullptr;
  CUDA_TRY(h, launch_export_fields(g, box_table(h), h->macro_valid ? h->rho + base : nullptr,
                                   h->macro_valid ? h->u + 3 * base : nullptr, as_double, B0,
                                   rho0, u0, d_solid, d_rho, d_u, h->stream));
  if (solid) CUDA_TRY(h, cudaMemcpyAsync(solid, d_solid, b_solid, cudaMemcpyDeviceToHost, h->stream));
  if (rho) CUDA_TRY(h, cudaMemcpyAsync(rho, d_rho, b_rho, cudaMemcpyDeviceToHost, h->stream));
  if (u) CUDA_TRY(h, cudaMemcpyAsync(u, d_u, b_u, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return LBMPSM_OK;
}

// ---------------------------------------------------------------------------
// Adjoint and tangent of the time-averaged drag (lbmpsm_adjoint_drag,
// lbmpsm_tangent_drag).
//
// Both calls run nsteps ordinary coupling steps with one fixed set of
// particle images -- the same map / collide / reduce launches as nsteps
// lbmpsm_step calls, so the lattice ends where those calls would leave it and
// J is the average of the forces they would return -- and differentiate
//   J = 1/M sum_{t=t0..t1} sum_images d . F_image(t),   M = t1 - t0 + 1,
// with respect to tau, Fext and the image centres (kernels in adjoint.cu).
//
// The adjoint keeps the state before every checkpoint_every-th step in HBM
// during the forward pass; the reverse pass recomputes each segment's states
// from its checkpoint (out-of-place FP64 collides into a segment store) and
// walks the segment backwards.  The tangent runs beside the forward pass.
namespace {

struct AdjScratch {
  std::vector<void*> blocks;
  ~AdjScratch() {
    for (void* p : blocks) cudaFree(p);
  }
  template <typename T>
  cudaError_t get(T** p, size_t bytes) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e == cudaSuccess) {
      blocks.push_back(q);
      *p = static_cast<T*>(q);
    }
    return e;
  }
};

int adj_validate(lbmpsm_handle* h, int n, const int* tag, const double* x, const double* v,
                 const double* omega, const double* radius, int nsteps, int t0, int t1,
                 const double* direction, double centre_step, const char* who) {
  const std::string w = who;
  if (h->opt.storage != LBMPSM_STORAGE_FP64)
    return fail(h, LBMPSM_ERR_STATE, w + ": the adjoint and tangent run on FP64 storage");
  if (h->nbox > 1) return fail(h, LBMPSM_ERR_STATE, w + ": needs a lattice of one box");
  if (!h->faces.empty())
    return fail(h, LBMPSM_ERR_STATE, w + ": needs a lattice without boundary conditions");
  for (int d = 0; d < h->g.dim; ++d)
    if (!h->prm.periodic[d])
      return fail(h, LBMPSM_ERR_STATE, w + ": needs a fully periodic lattice");
  if (n < 0 || nsteps < 1 || t0 < 1 || t1 < t0 || t1 > nsteps)
    return fail(h, LBMPSM_ERR_ARG, w + ": needs 1 <= t0 <= t1 <= nsteps and n >= 0");
  if (n > 0 && (!tag || !x || !v || !omega || !radius))
    return fail(h, LBMPSM_ERR_ARG, w + ": NULL particle array");
  if (!direction || !std::isfinite(direction[0]) || !std::isfinite(direction[1]) ||
      !std::isfinite(direction[2]))
    return fail(h, LBMPSM_ERR_ARG, w + ": the drag direction must be finite");
  if (!(centre_step > 0.0) || !std::isfinite(centre_step))
    return fail(h, LBMPSM_ERR_ARG, w + ": centre_step must be positive");
  return LBMPSM_OK;
}

int adj_alloc_nodes(lbmpsm_handle* h, AdjScratch& sc, AdjNodes& an) {
  const size_t N = (size_t)h->g.N;
  CUDA_TRY(h, sc.get(&an.band, N));
  CUDA_TRY(h, sc.get(&an.tag, sizeof(int2) * N));
  CUDA_TRY(h, sc.get(&an.us, sizeof(double) * 6 * N));
  CUDA_TRY(h, sc.get(&an.cw, sizeof(int2) * N));
  CUDA_TRY(h, sc.get(&an.sigma, sizeof(double) * 2 * N));
  CUDA_TRY(h, sc.get(&an.edot, sizeof(double) * 2 * N));
  CUDA_TRY(h, cudaMemsetAsync(an.band, 0, N, h->stream));
  CUDA_TRY(h, cudaMemsetAsync(an.tag, 0, sizeof(int2) * N, h->stream));
  CUDA_TRY(h, cudaMemsetAsync(an.us, 0, sizeof(double) * 6 * N, h->stream));
  CUDA_TRY(h, cudaMemsetAsync(an.cw, 0, sizeof(int2) * N, h->stream));
  CUDA_TRY(h, cudaMemsetAsync(an.sigma, 0, sizeof(double) * 2 * N, h->stream));
  CUDA_TRY(h, cudaMemsetAsync(an.edot, 0, sizeof(double) * 2 * N, h->stream));
  return LBMPSM_OK;
}

// slot entries and count weights from the table and the cell lists of the map
// that just ran (n > 0)
int adj_entries(lbmpsm_handle* h, const AdjNodes& an, int n, double centre_step) {
  if (n == 0) return LBMPSM_OK;
  AdjSetup s{};
  s.g = h->g;
  s.tab = h->tab;
  s.an = an;
  s.img = h->d_img;
  s.n = n;
  const int ncells = h->C[0] * h->C[1] * h->C[2];
  s.cell_count = h->d_cells;
  s.cell_off = h->d_cells + ncells;
  s.list = h->d_list;
  for (int d = 0; d < 3; ++d) {
    s.cb[d] = h->cb[d];
    s.C[d] = h->C[d];
  }
  s.h0 = h->g.dim == 3 ? std::sqrt(3.1) / 2.0 : std::sqrt(2.1) / 2.0;
  s.hl = centre_step / h->dx;
  s.status = h->d_status;
  CUDA_TRY(h, launch_adj_entries(s, h->stream));
  return LBMPSM_OK;
}

AdjParams adj_params(const lbmpsm_handle* h, const AdjNodes& an, double* part,
                     const double* direction) {
  AdjParams p{};
  p.g = h->g;
  p.tab = h->tab;
  p.bp = h->boxes[0];
  p.weighting = h->opt.psm_weighting;
  p.an = an;
  p.part = part;
  for (int d = 0; d < 3; ++d) p.d[d] = direction[d];
  return p;
}

AdjCentre adj_centre(const lbmpsm_handle* h, const AdjNodes& an, int n, double centre_step) {
  AdjCentre c{};
  c.g = h->g;
  c.tab = h->tab;
  c.an = an;
  c.img = h->d_img;
  c.n = n;
  c.x = h->d_xvw;
  for (int d = 0; d < 3; ++d) c.origin[d] = h->boxes[0].origin[d];
  c.dx = h->dx;
  c.h = centre_step;
  c.h0 = h->g.dim == 3 ? std::sqrt(3.1) / 2.0 : std::sqrt(2.1) / 2.0;
  c.tau = h->boxes[0].tau;
  c.weighting = h->opt.psm_weighting;
  return c;
}

// one out-of-place FP64 collide (no macro store): dst = step(src) at parity odd
int collide_into(lbmpsm_handle* h, const double* src, double* dst, int odd) {
  CollideParams p{};
  p.g = h->g;
  p.f = dst;
  p.fsrc = src;
  p.tab = h->tab;
  p.weighting = h->opt.psm_weighting;
  p.box = h->d_box;
  p.has_force = h->any_force ? 1 : 0;
  p.invCs2 = h->invCs2;
  p.invCs4 = h->invCs4;
  p.status = h->d_status;
  CUDA_TRY(h, launch_collide_f64(p, odd, h->stream));
  return LBMPSM_OK;
}

int adj_status(lbmpsm_handle* h, const char* who) {
  int st = 0;
  CUDA_TRY(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  if (st & (STATUS_ADJ_CROWDED | STATUS_ADJ_SAME_TAG)) {
    CUDA_TRY(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return fail(h, LBMPSM_ERR_ARG,
                std::string(who) +
                    ((st & STATUS_ADJ_CROWDED)
                         ? ": a node lies in the surface shells of more than two particles"
                         : ": two images of one particle share a surface node"));
  }
  return read_status(h);
}

}  // namespace

extern "C" {

int lbmpsm_adjoint_drag(lbmpsm_handle* h, int n, const int* tag, const double* x,
                        const double* v, const double* omega, const double* radius, int nsteps,
                        int t0, int t1, const double* direction, int checkpoint_every,
                        double centre_step, double* J, double* dJ_dtau, double* dJ_dFext,
                        double* dJ_dx, double* drag_per_step) {
  if (!h) return LBMPSM_ERR_ARG;
  const char* who = "lbmpsm_adjoint_drag";
  int rc = adj_validate(h, n, tag, x, v, omega, radius, nsteps, t0, t1, direction, centre_step, who);
  if (rc) return rc;
  if (checkpoint_every < 1) return fail(h, LBMPSM_ERR_ARG, std::string(who) + ": checkpoint_every must be >= 1");
  if (n > 0 && !dJ_dx) return fail(h, LBMPSM_ERR_ARG, std::string(who) + ": dJ_dx is NULL");
  rc = stage_images(h, n, nullptr, tag, x, v, omega, radius);
  if (rc) return rc;
  const int T = nsteps, K = std::min(checkpoint_every, nsteps);
  const int nseg = (T + K - 1) / K;
  const size_t state = sizeof(double) * (size_t)h->g.Np * h->g.Q;
  const size_t nstates = (size_t)nseg + (size_t)(K - 1) + 2;
  {
    size_t fr = 0, tot = 0;
    CUDA_TRY(h, cudaMemGetInfo(&fr, &tot));
    const size_t need = nstates * state + (size_t)h->g.N * 88;
    if (need + (size_t)(256u << 20) > fr)
      return fail(h, LBMPSM_ERR_NOMEM,
                  std::string(who) + ": checkpoints and the segment store need " +
                      std::to_string(need) + " bytes of device memory, " + std::to_string(fr) +
                      " are free; choose checkpoint_every near sqrt(nsteps)");
  }
  AdjScratch sc;
  AdjNodes an{};
  rc = adj_alloc_nodes(h, sc, an);
  if (rc) return rc;
  const long long nb = adj_blocks(h->g);
  double *part = nullptr, *sums = nullptr, *drag = nullptr, *gx = nullptr;
  CUDA_TRY(h, sc.get(&part, sizeof(double) * ADJ_PART * (size_t)nb));
  CUDA_TRY(h, sc.get(&sums, sizeof(double) * ADJ_PART));
  CUDA_TRY(h, sc.get(&drag, sizeof(double) * (size_t)T));
  CUDA_TRY(h, sc.get(&gx, sizeof(double) * 3 * (size_t)std::max(n, 1)));
  CUDA_TRY(h, cudaMemsetAsync(part, 0, sizeof(double) * ADJ_PART * (size_t)nb, h->stream));
  CUDA_TRY(h, cudaMemsetAsync(drag, 0, sizeof(double) * (size_t)T, h->stream));
  CUDA_TRY(h, cudaMemsetAsync(gx, 0, sizeof(double) * 3 * (size_t)std::max(n, 1), h->stream));
  std::vector<double*> ckpt((size_t)nseg), store((size_t)std::max(K - 1, 0));
  for (auto& c : ckpt) CUDA_TRY(h, sc.get(&c, state));
  for (auto& c : store) CUDA_TRY(h, sc.get(&c, state));
  double* lam[2];
  for (auto& l : lam) CUDA_TRY(h, sc.get(&l, state));
  CUDA_TRY(h, cudaMemsetAsync(lam[0], 0, state, h->stream));

  // forward pass: the ordinary steps, a checkpoint before every K-th
  const long long ts = h->t;
  for (int t = 1; t <= T; ++t) {
    if ((t - 1) % K == 0)
      CUDA_TRY(h, cudaMemcpyAsync(ckpt[(size_t)((t - 1) / K)], h->f, state,
                                  cudaMemcpyDeviceToDevice, h->stream));
    rc = enqueue_step(h, n);
    if (rc) return rc;
    if (t == 1) {
      rc = adj_entries(h, an, n, centre_step);
      if (rc) return rc;
    }
    if (n > 0)
      CUDA_TRY(h, launch_adj_drag(h->d_out, n, direction[0], direction[1], direction[2],
                                  drag + (t - 1), h->stream));
  }
  rc = adj_status(h, who);
  if (rc) return rc;

  // reverse pass, segment by segment
  const double cwin = h->forceFactor / (double)(t1 - t0 + 1);
  AdjParams p = adj_params(h, an, part, direction);
  int cur = 0;  // lam[cur] holds lambda of the step after the one being reversed
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int a = seg * K + 1, b = std::min(a + K - 1, T);
    auto st_of = [&](int t) { return t == a ? ckpt[(size_t)seg] : store[(size_t)(t - a - 1)]; };
    for (int t = a + 1; t <= b; ++t) {
      rc = collide_into(h, st_of(t - 1), st_of(t), (int)((ts + t - 2) & 1));
      if (rc) return rc;
    }
    for (int t = b; t >= a; --t) {
      p.state = st_of(t);
      p.odd = (int)((ts + t - 1) & 1);
      p.lin = lam[cur];
      p.lout = lam[cur ^ 1];
      p.c = (t >= t0 && t <= t1) ? cwin : 0.0;
      CUDA_TRY(h, launch_adj_step(p, 0, h->stream));
      cur ^= 1;
    }
  }
  AdjCentre c = adj_centre(h, an, n, centre_step);
  c.out = gx;
  CUDA_TRY(h, launch_adj_centre(c, h->stream));
  CUDA_TRY(h, launch_adj_sum(part, nb, sums, h->stream));
  std::vector<double> hd((size_t)T), hs(ADJ_PART), hx(3 * (size_t)std::max(n, 1));
  CUDA_TRY(h, cudaMemcpyAsync(hd.data(), drag, sizeof(double) * (size_t)T, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(hs.data(), sums, sizeof(double) * ADJ_PART, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(hx.data(), gx, sizeof(double) * hx.size(), cudaMemcpyDeviceToHost, h->stream));
  rc = adj_status(h, who);  // synchronises
  if (rc) return rc;
  double sJ = 0.0;
  for (int t = t0; t <= t1; ++t) sJ += hd[(size_t)(t - 1)];
  const double omega_lb = h->boxes[0].omega;
  if (J) *J = sJ / (double)(t1 - t0 + 1);
  if (dJ_dtau) *dJ_dtau = -omega_lb * omega_lb * hs[0] + hs[1];
  if (dJ_dFext)
    for (int d = 0; d < 3; ++d) dJ_dFext[d] = hs[2 + d] / h->volumeForceFactor;
  if (n > 0) std::memcpy(dJ_dx, hx.data(), sizeof(double) * 3 * (size_t)n);
  if (drag_per_step) std::memcpy(drag_per_step, hd.data(), sizeof(double) * (size_t)T);
  return LBMPSM_OK;
}

int lbmpsm_tangent_drag(lbmpsm_handle* h, int n, const int* tag, const double* x,
                        const double* v, const double* omega, const double* radius, int nsteps,
                        int t0, int t1, const double* direction, double centre_step,
                        double dtau, const double* dFext, const double* dx, double* J,
                        double* dJ) {
  if (!h) return LBMPSM_ERR_ARG;
  const char* who = "lbmpsm_tangent_drag";
  int rc = adj_validate(h, n, tag, x, v, omega, radius, nsteps, t0, t1, direction, centre_step, who);
  if (rc) return rc;
  if (!std::isfinite(dtau) || (dFext && !finite_all(dFext, 3)) ||
      (dx && n > 0 && !finite_all(dx, 3 * (size_t)n)))
    return fail(h, LBMPSM_ERR_ARG, std::string(who) + ": the direction must be finite");
  rc = stage_images(h, n, nullptr, tag, x, v, omega, radius);
  if (rc) return rc;
  const int T = nsteps;
  const size_t state = sizeof(double) * (size_t)h->g.Np * h->g.Q;
  AdjScratch sc;
  AdjNodes an{};
  rc = adj_alloc_nodes(h, sc, an);
  if (rc) return rc;
  const long long nb = adj_blocks(h->g);
  double *part = nullptr, *sums = nullptr, *drag = nullptr, *xdot = nullptr, *s1 = nullptr;
  double* tng[2];
  CUDA_TRY(h, sc.get(&part, sizeof(double) * ADJ_PART * (size_t)nb));
  CUDA_TRY(h, sc.get(&sums, sizeof(double) * ADJ_PART));
  CUDA_TRY(h, sc.get(&drag, sizeof(double) * (size_t)T));
  CUDA_TRY(h, sc.get(&xdot, sizeof(double) * 3 * (size_t)std::max(n, 1)));
  CUDA_TRY(h, sc.get(&s1, state));
  for (auto& t : tng) CUDA_TRY(h, sc.get(&t, state));
  CUDA_TRY(h, cudaMemsetAsync(part, 0, sizeof(double) * ADJ_PART * (size_t)nb, h->stream));
  CUDA_TRY(h, cudaMemsetAsync(drag, 0, sizeof(double) * (size_t)T, h->stream));
  CUDA_TRY(h, cudaMemsetAsync(tng[0], 0, state, h->stream));
  std::vector<double> hxd(3 * (size_t)std::max(n, 1), 0.0);
  if (dx && n > 0) std::memcpy(hxd.data(), dx, sizeof(double) * 3 * (size_t)n);
  CUDA_TRY(h, cudaMemcpyAsync(xdot, hxd.data(), sizeof(double) * hxd.size(), cudaMemcpyHostToDevice,
                              h->stream));

  AdjParams p = adj_params(h, an, part, direction);
  const double omega_lb = h->boxes[0].omega;
  p.dtau = dtau;
  p.domega = -omega_lb * omega_lb * dtau;
  for (int d = 0; d < 3; ++d) p.dF[d] = dFext ? dFext[d] / h->volumeForceFactor : 0.0;
  const double cwin = h->forceFactor / (double)(t1 - t0 + 1);
  const long long ts = h->t;
  int cur = 0;
  for (int t = 1; t <= T; ++t) {
    // the tangent step reads the state before this step's collide; the table
    // it needs exists after the first map, so step 1 runs from a copy
    if (t == 1) CUDA_TRY(h, cudaMemcpyAsync(s1, h->f, state, cudaMemcpyDeviceToDevice, h->stream));
    if (t > 1) {
      p.state = static_cast<const double*>(h->f);
      p.odd = (int)((ts + t - 1) & 1);
      p.lin = tng[cur];
      p.lout = tng[cur ^ 1];
      p.c = (t >= t0 && t <= t1) ? cwin : 0.0;
      CUDA_TRY(h, launch_adj_step(p, 1, h->stream));
      cur ^= 1;
    }
    rc = enqueue_step(h, n);
    if (rc) return rc;
    if (t == 1) {
      rc = adj_entries(h, an, n, centre_step);
      if (rc) return rc;
      AdjCentre c = adj_centre(h, an, n, centre_step);
      c.xdot = xdot;
      CUDA_TRY(h, launch_adj_centre(c, h->stream));
      p.state = s1;
      p.odd = (int)(ts & 1);
      p.lin = tng[cur];
      p.lout = tng[cur ^ 1];
      p.c = (t >= t0 && t <= t1) ? cwin : 0.0;
      CUDA_TRY(h, launch_adj_step(p, 1, h->stream));
      cur ^= 1;
    }
    if (n > 0)
      CUDA_TRY(h, launch_adj_drag(h->d_out, n, direction[0], direction[1], direction[2],
                                  drag + (t - 1), h->stream));
  }
  CUDA_TRY(h, launch_adj_sum(part, nb, sums, h->stream));
  std::vector<double> hd((size_t)T), hs(ADJ_PART);
  CUDA_TRY(h, cudaMemcpyAsync(hd.data(), drag, sizeof(double) * (size_t)T, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(hs.data(), sums, sizeof(double) * ADJ_PART, cudaMemcpyDeviceToHost, h->stream));
  rc = adj_status(h, who);
  if (rc) return rc;
  double sJ = 0.0;
  for (int t = t0; t <= t1; ++t) sJ += hd[(size_t)(t - 1)];
  if (J) *J = sJ / (double)(t1 - t0 + 1);
  if (dJ) *dJ = hs[0];
  return LBMPSM_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Groups of lattices stepped as one CUDA graph (lbmpsm_group_*).
//
// A batched ensemble holds boxes of one lattice geometry; boxes of different
// sizes form separate handles.  A group advances several handles together:
// one step of every member (map, collide, reduce, boundary condition, each
// on the member's own streams as lbmpsm_run_fixed would run it) is captured
// once per A-A parity into a single graph whose branches run concurrently,
// so that all members take one graph launch per step.
struct lbmpsm_group {
  std::vector<lbmpsm_handle*> hs;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr, fork2 = nullptr;
  std::vector<cudaEvent_t> join, join2;
  cudaGraphExec_t gexec[2]{nullptr, nullptr};
  std::vector<long long> gen;  // members' graph generations the graphs were captured at
  std::vector<int> cap_n, cap_bc;
  std::string err;
  // one collide launch for every member (when they qualify): the member
  // table in device memory and the launch shape
  bool fused = false;
  MultiMember* d_members = nullptr;
  std::vector<MultiMember> members;
  MultiCollide mc{};
  // which plan the graphs take: -1 = not yet timed (one launch when the
  // members qualify), 0 = one collide per member, 1 = one launch for all;
  // the group's tuner times both on live steps (their results are
  // bit-identical) and keeps the faster
  int plan_pref = -1;
  bool tuned = false;
  float tune_ms[2] = {-1.f, -1.f};  // ms per step: [0] per member, [1] one launch
  cudaEvent_t t0 = nullptr, t1 = nullptr;
};

namespace {
int gfail(lbmpsm_group* g, int code, const std::string& msg) {
  g->err = msg;
  return code;
}
#define GROUP_TRY(g, call)                                                                  \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return gfail((g), LBMPSM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

void group_drop(lbmpsm_group* g) {
  for (int k = 0; k < 2; ++k)
    if (g->gexec[k]) {
      cudaGraphExecDestroy(g->gexec[k]);
      g->gexec[k] = nullptr;
    }
}

// Whether the members' collides run as one launch, and if so its member
// table and shape.  The members must be 3-D and periodic on every axis,
// share storage precision and PSM weighting, and either all have a body
// force or none; at most MULTI_MAX members; the row pipeline takes rows of
// up to 128 nodes.  LBMPSM_GROUP_FUSE=0 keeps one collide per member.
// whether the members qualify for one collide launch
bool group_fusable(const lbmpsm_group* g) {
  const size_t m = g->hs.size();
  if (m > (size_t)MULTI_MAX || !g->d_members) return false;
  const lbmpsm_handle* h0 = g->hs[0];
  for (const lbmpsm_handle* h : g->hs) {
    if (h->g.dim != 3 || h->opt.storage != h0->opt.storage ||
        h->opt.psm_weighting != h0->opt.psm_weighting || h->any_force != h0->any_force)
      return false;
    for (int d = 0; d < 3; ++d)
      if (!h->g.per[d]) return false;
  }
  return true;
}

int group_plan_collide(lbmpsm_group* g) {
  g->fused = false;
  const char* env = std::getenv("LBMPSM_GROUP_FUSE");
  if (env && std::atoi(env) == 0) return LBMPSM_OK;
  if (g->plan_pref == 0 && !(env && std::atoi(env) == 1)) return LBMPSM_OK;
  if (!group_fusable(g)) return LBMPSM_OK;
  const size_t m = g->hs.size();
  const lbmpsm_handle* h0 = g->hs[0];
  g->members.assign(m, MultiMember{});
  for (size_t i = 0; i < m; ++i) {
    g->members[i].p = collide_params(g->hs[i]);
    g->members[i].p.store_macro = 0;
    g->members[i].has_force = g->hs[i]->any_force ? 1 : 0;
  }
  MultiCollide mc{};
  mc.m = g->d_members;
  mc.nm = (int)m;
  mc.any_force = h0->any_force ? 1 : 0;
  mc.status = g->hs[0]->d_status;
  mc.full_wait_limit = g->hs[0]->full_wait_limit;
  if (prepare_collide_multi(mc, g->members.data(), h0->opt.storage, h0->sm_count) != cudaSuccess) {
    cudaGetLastError();
    return LBMPSM_OK;  // (rows too wide, or too many tiles): one collide per member
  }
  // ordered after the group's earlier launches, which may still read the table
  GROUP_TRY(g, cudaMemcpyAsync(g->d_members, g->members.data(), sizeof(MultiMember) * m,
                               cudaMemcpyHostToDevice, g->stream));
  GROUP_TRY(g, cudaStreamSynchronize(g->stream));
  g->mc = mc;
  g->fused = true;
  return LBMPSM_OK;
}

// Capture the graph of one step of every member for parity par.
int group_capture(lbmpsm_group* g, int par) {
  const size_t m = g->hs.size();
  cudaGraph_t graph = nullptr;
  std::vector<long long> t0(m);
  for (size_t i = 0; i < m; ++i) t0[i] = g->hs[i]->t;
  if (!g->gexec[par ^ 1]) {  // planned once for both parities' graphs
    const int prc = group_plan_collide(g);
    if (prc) return prc;
  }
  GROUP_TRY(g, cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
  int rc = LBMPSM_OK;
  cudaError_t ce = cudaEventRecord(g->fork, g->stream);
  if (!g->fused) {
    // each member's whole step as one branch
    for (size_t i = 0; i < m && !rc && ce == cudaSuccess; ++i) {
      lbmpsm_handle* h = g->hs[i];
      ce = cudaStreamWaitEvent(h->stream, g->fork, 0);
      if (ce != cudaSuccess) break;
      rc = enqueue_step(h, h->last_n, true);
      if (rc) rc = gfail(g, rc, h->err);
      if (!rc) ce = cudaEventRecord(g->join[i], h->stream);
      if (!rc && ce == cudaSuccess) ce = cudaStreamWaitEvent(g->stream, g->join[i], 0);
    }
  } else {
    // the members' maps as branches, one collide launch for all members,
    // then their boundary faces and reductions as branches
    for (size_t i = 0; i < m && !rc && ce == cudaSuccess; ++i) {
      lbmpsm_handle* h = g->hs[i];
      ce = cudaStreamWaitEvent(h->stream, g->fork, 0);
      if (ce != cudaSuccess) break;
      rc = enqueue_map(h, h->last_n);
      if (rc) rc = gfail(g, rc, h->err);
      if (!rc) ce = cudaEventRecord(g->join[i], h->stream);
      if (!rc && ce == cudaSuccess) ce = cudaStreamWaitEvent(g->stream, g->join[i], 0);
    }
    if (!rc && ce == cudaSuccess)
      ce = launch_collide_multi(g->mc, g->hs[0]->opt.storage, par, g->stream);
    if (!rc && ce == cudaSuccess) {
      for (size_t i = 0; i < m; ++i) collide_done(g->hs[i]);
      ce = cudaEventRecord(g->fork2, g->stream);
    }
    for (size_t i = 0; i < m && !rc && ce == cudaSuccess; ++i) {
      lbmpsm_handle* h = g->hs[i];
      ce = cudaStreamWaitEvent(h->stream, g->fork2, 0);
      if (ce != cudaSuccess) break;
      rc = enqueue_post(h, h->last_n, true);
      if (rc) rc = gfail(g, rc, h->err);
      if (!rc) ce = cudaEventRecord(g->join2[i], h->stream);
      if (!rc && ce == cudaSuccess) ce = cudaStreamWaitEvent(g->stream, g->join2[i], 0);
    }
  }
  cudaError_t ee = cudaStreamEndCapture(g->stream, &graph);
  for (size_t i = 0; i < m; ++i) g->hs[i]->t = t0[i];  // captured, not run
  if (rc || ce != cudaSuccess || ee != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    if (rc) return rc;
    GROUP_TRY(g, ce);
    GROUP_TRY(g, ee);
  }
  cudaError_t ie = cudaGraphInstantiate(&g->gexec[par], graph, 0);
  cudaGraphDestroy(graph);
  GROUP_TRY(g, ie);
  g->gen.resize(m);
  g->cap_n.resize(m);
  g->cap_bc.resize(m);
  for (size_t i = 0; i < m; ++i) {
    g->gen[i] = g->hs[i]->graph_gen;
    g->cap_n[i] = g->hs[i]->last_n;
    g->cap_bc[i] = g->hs[i]->faces.empty() ? 0 : 1;
  }
  return LBMPSM_OK;
}

// One step of the group: its graph for the members' parity (captured on
// first use), launched on the group's stream.
int group_step(lbmpsm_group* g) {
  const int par = (int)(g->hs[0]->t & 1);
  if (!g->gexec[par]) {
    const int rc = group_capture(g, par);
    if (rc) return rc;
  }
  GROUP_TRY(g, cudaGraphLaunch(g->gexec[par], g->stream));
  for (lbmpsm_handle* h : g->hs) h->t += 1;
  return LBMPSM_OK;
}
}  // namespace

extern "C" {

int lbmpsm_group_create(lbmpsm_handle* const* handles, int count, lbmpsm_group** out) {
  if (!out) return LBMPSM_ERR_ARG;
  *out = nullptr;
  if (!handles || count < 1) return fail(nullptr, LBMPSM_ERR_ARG, "a group needs at least one lattice");
  for (int i = 0; i < count; ++i) {
    if (!handles[i]) return fail(nullptr, LBMPSM_ERR_ARG, "NULL lattice in a group");
    if (handles[i]->device != handles[0]->device)
      return fail(nullptr, LBMPSM_ERR_ARG, "the lattices of a group must be on one device");
    for (int j = 0; j < i; ++j)
      if (handles[j] == handles[i])
        return fail(nullptr, LBMPSM_ERR_ARG, "a lattice appears twice in a group");
  }
  lbmpsm_group* g = new (std::nothrow) lbmpsm_group();
  if (!g) return fail(nullptr, LBMPSM_ERR_NOMEM, "host allocation failed");
  g->hs.assign(handles, handles + count);
  g->device = handles[0]->device;
  g->join.assign((size_t)count, nullptr);
  g->join2.assign((size_t)count, nullptr);
  bool ok = cudaSetDevice(g->device) == cudaSuccess &&
            cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&g->fork2, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming) == cudaSuccess;
  for (auto& e : g->join) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  for (auto& e : g->join2) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  ok = ok && cudaMalloc(&g->d_members, sizeof(MultiMember) * MULTI_MAX) == cudaSuccess;
  ok = ok && cudaEventCreate(&g->t0) == cudaSuccess && cudaEventCreate(&g->t1) == cudaSuccess;
  if (!ok) {
    lbmpsm_group_destroy(g);
    return fail(nullptr, LBMPSM_ERR_CUDA, "group set-up failed");
  }
  *out = g;
  return LBMPSM_OK;
}

void lbmpsm_group_destroy(lbmpsm_group* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  group_drop(g);
  for (auto e : g->join)
    if (e) cudaEventDestroy(e);
  for (auto e : g->join2)
    if (e) cudaEventDestroy(e);
  if (g->fork2) cudaEventDestroy(g->fork2);
  if (g->t0) cudaEventDestroy(g->t0);
  if (g->t1) cudaEventDestroy(g->t1);
  if (g->d_members) cudaFree(g->d_members);
  if (g->fork) cudaEventDestroy(g->fork);
  if (g->done) cudaEventDestroy(g->done);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

const char* lbmpsm_group_last_error(const lbmpsm_group* g) { return g ? g->err.c_str() : ""; }

void* lbmpsm_group_stream(lbmpsm_group* g) { return g ? (void*)g->stream : nullptr; }

int lbmpsm_group_tune_ms(const lbmpsm_group* g, float* ms) {
  if (!g || !ms) return LBMPSM_ERR_ARG;
  ms[0] = g->tune_ms[0];
  ms[1] = g->tune_ms[1];
  return LBMPSM_OK;
}

int lbmpsm_group_collide_launches(const lbmpsm_group* g) {
  if (!g || (!g->gexec[0] && !g->gexec[1])) return -1;
  return g->fused ? 1 : (int)g->hs.size();
}

int lbmpsm_group_run_fixed(lbmpsm_group* g, int nsteps) {
  if (!g || nsteps < 0) return LBMPSM_ERR_ARG;
  GROUP_TRY(g, cudaSetDevice(g->device));
  const size_t m = g->hs.size();
  const long long par0 = g->hs[0]->t & 1;
  for (size_t i = 0; i < m; ++i) {
    lbmpsm_handle* h = g->hs[i];
    if ((h->t & 1) != par0)
      return gfail(g, LBMPSM_ERR_STATE, "the lattices of a group must be at the same step parity");
    if (h->macro_requested)
      return gfail(g, LBMPSM_ERR_STATE, "a member has a macro-field store pending (use lbmpsm_run_fixed)");
    const int rc = maybe_tune(h);
    if (rc) return gfail(g, rc, h->err);
  }
  // the graphs are stale if a member's buffers, images or boundary condition changed
  bool stale = g->gen.size() != m;
  for (size_t i = 0; !stale && i < m; ++i) {
    const lbmpsm_handle* h = g->hs[i];
    stale = g->gen[i] != h->graph_gen || g->cap_n[i] != h->last_n ||
            g->cap_bc[i] != (h->faces.empty() ? 0 : 1);
  }
  if (stale) group_drop(g);
  // order after the members' earlier work
  for (size_t i = 0; i < m; ++i) {
    GROUP_TRY(g, cudaEventRecord(g->join[i], g->hs[i]->stream));
    GROUP_TRY(g, cudaStreamWaitEvent(g->stream, g->join[i], 0));
  }
  // the group's tuner: with at least 8 steps to run and members that qualify
  // for one collide launch, time two steps of each plan (after two untimed
  // steps that capture its graphs) and keep the faster
  const char* fenv = std::getenv("LBMPSM_GROUP_FUSE");
  if (!g->tuned && nsteps >= 8 && !fenv && group_fusable(g)) {
    g->tuned = true;
    for (int plan = 1; plan >= 0; --plan) {
      group_drop(g);
      g->plan_pref = plan;
      for (int k = 0; k < 2; ++k) {
        const int rc = group_step(g);
        if (rc) return rc;
      }
      GROUP_TRY(g, cudaEventRecord(g->t0, g->stream));
      for (int k = 0; k < 2; ++k) {
        const int rc = group_step(g);
        if (rc) return rc;
      }
      GROUP_TRY(g, cudaEventRecord(g->t1, g->stream));
      GROUP_TRY(g, cudaEventSynchronize(g->t1));
      float ms = 0.f;
      GROUP_TRY(g, cudaEventElapsedTime(&ms, g->t0, g->t1));
      g->tune_ms[plan] = ms / 2;
      nsteps -= 4;
    }
    const int best = g->tune_ms[1] <= g->tune_ms[0] ? 1 : 0;
    if (best != g->plan_pref) group_drop(g);
    g->plan_pref = best;
  }
  for (int s = 0; s < nsteps; ++s) {
    const int rc = group_step(g);
    if (rc) return rc;
  }
  // the members' later work is ordered after the group's
  GROUP_TRY(g, cudaEventRecord(g->done, g->stream));
  for (size_t i = 0; i < m; ++i) GROUP_TRY(g, cudaStreamWaitEvent(g->hs[i]->stream, g->done, 0));
  return LBMPSM_OK;
}

}  // extern "C"
