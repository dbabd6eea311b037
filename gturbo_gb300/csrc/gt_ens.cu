// gt_ens.cu -- batched ensembles and the Philox forcing.
//
// An ensemble advances many independent fields (members) that may differ in grid size
// (128 ... 2048), alpha, time step and forcing. One launch per pass covers every member: each
// CTA reads its (member, tile) work item and runs the same tile functions as the single-field
// kernels, so a member's results are bit-identical to advancing it alone. One step (all RK
// stages + the forcing of every member) is captured once as a CUDA graph on the ensemble's
// own stream and replayed. Every member has its own counter-based Philox forcing stream:
// the phase of mode k at step s is a function of (key, s, k) only, so all modes of all
// members are drawn in parallel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/gturbo.h"
#include "gt_internal.h"
#include "gt_ens_kernels.cuh"
#include "gt_philox.h"

namespace gt {

struct ForceMember {
  double2* z;
  const int* ikx;
  const int* iky;
  const int* jc;
  int nf;
  int nh;
  double sf;      // sqrt(dt) * famp
  uint64_t key;   // Philox stream of the member
};

// One kick of mode k (the reference's forcing.f90:21-31 with a Philox phase): the mode gets
// sf (cos te, sin te), its conjugate partner on the kx=0 / Nyquist columns sf (cos te, -sin te).
__device__ __forceinline__ void philox_kick(const ForceMember& m, int k, uint64_t step) {
  const double te = philox_phase(m.key, step, (uint64_t)k);
  double sn, cs;
  sincos(te, &sn, &cs);
  const int i = m.ikx[k], j = m.iky[k];
  double2* p = m.z + (size_t)j * m.nh + i;
  double2 a = *p;
  a.x = a.x + m.sf * cs;
  a.y = a.y + m.sf * sn;
  *p = a;
  if (i == 0 || i == m.nh - 1) {
    double2* pc = m.z + (size_t)m.jc[j] * m.nh + i;
    double2 b = *pc;
    b.x = b.x + m.sf * cs;
    b.y = b.y - m.sf * sn;
    *pc = b;
  }
}

__global__ void k_forcing_philox1(ForceMember m, uint64_t step) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m.nf) philox_kick(m, k, step);
}

// Every member's kick; the step counter lives on the device and the last block to finish
// advances it (after every block has read it), so a replayed graph draws fresh phases.
__global__ void k_forcing_philox_ens(const ForceMember* __restrict__ fm, const int2* __restrict__ modes,
                                     int total, uint64_t* step_ctr, unsigned* done) {
  const uint64_t step = *step_ctr;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < total) {
    const int2 mk = modes[g];
    const ForceMember m = fm[mk.x];
    philox_kick(m, mk.y, step);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned t = atomicAdd(done, 1u);
    if (t == gridDim.x - 1) {
      *done = 0u;
      *step_ctr = step + 1;
      __threadfence();
    }
  }
}

}  // namespace gt

using gt::EnsTile;
using gt::ForceMember;
using gt::NltArgs;

struct gt_ens {
  int nm = 0, rko = 2, stages = 2;
  std::vector<gt_params> params;
  std::vector<uint64_t> keys;
  std::vector<gt_handle*> handles;  // one per distinct parameter set
  std::vector<int> hidx;            // member -> handle
  std::vector<double*> z, znl, znew, u, v;
  bool fields_set = false;
  NltArgs* d_args = nullptr;        // [stages][nm]
  EnsTile* d_col = nullptr;
  EnsTile* d_row = nullptr;
  int ncol = 0, nrow = 0;
  int* d_flags = nullptr;
  ForceMember* d_fm = nullptr;
  int2* d_modes = nullptr;
  int nmodes = 0;
  uint64_t* d_step = nullptr;
  unsigned* d_done = nullptr;
  cudaStream_t user = nullptr, own = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool use_graph = true;
  int tile_r = 8;  // values per thread of the pass kernels (tile family 16, 8 or 4)
  std::string err;
};

namespace {

int efail(gt_ens* e, int code, const std::string& msg) {
  if (e) e->err = msg;
  else gt::set_error(nullptr, code, msg.c_str());
  return code;
}

int ecuda(gt_ens* e, cudaError_t c, const char* what) {
  return efail(e, GT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(c));
}

#define GE_CUDA(e, call)                                  \
  do {                                                    \
    cudaError_t c_ = (call);                              \
    if (c_ != cudaSuccess) return ecuda(e, c_, #call);    \
  } while (0)

void drop_graph(gt_ens* e) {
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  if (e->graph) cudaGraphDestroy(e->graph);
  e->gexec = nullptr;
  e->graph = nullptr;
}

void free_ens(gt_ens* e) {
  drop_graph(e);
  void* ptrs[] = {e->d_args, e->d_col, e->d_row, e->d_flags, e->d_fm, e->d_modes, e->d_step, e->d_done};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (e->own) cudaStreamDestroy(e->own);
  if (e->ev_in) cudaEventDestroy(e->ev_in);
  if (e->ev_out) cudaEventDestroy(e->ev_out);
  for (gt_handle* h : e->handles) gt_destroy(h);
}

bool valid_ens_n(int n) { return n >= 128 && n <= 2048 && (n & (n - 1)) == 0; }

// the launch parameters of one step's passes (gt_ens_kernels.cuh)
gt::EnsLaunch ens_launch(const gt_ens* e) {
  return gt::EnsLaunch{e->ncol, e->nrow, e->stages, e->nm, e->d_args, e->d_col, e->d_row};
}

int enqueue_step(gt_ens* e, cudaStream_t s) {
  if (e->tile_r == 16) gt::ens_passes_r16(ens_launch(e), s);
  else if (e->tile_r == 4) gt::ens_passes_r4(ens_launch(e), s);
  else gt::ens_passes_r8(ens_launch(e), s);
  if (e->nmodes > 0)
    gt::k_forcing_philox_ens<<<(e->nmodes + 127) / 128, 128, 0, s>>>(e->d_fm, e->d_modes, e->nmodes,
                                                                    e->d_step, e->d_done);
  cudaError_t c = cudaGetLastError();
  return c == cudaSuccess ? GT_OK : ecuda(e, c, "ensemble launch");
}

}  // namespace

extern "C" {

int gt_ens_create(const gt_params* members, int32_t nmembers, const uint64_t* keys, gt_ens** out) {
  if (!members || !keys || !out || nmembers < 1)
    return efail(nullptr, GT_ERR_ARG, "gt_ens_create: null argument or no member");
  *out = nullptr;
  gt_ens* e = new (std::nothrow) gt_ens();
  if (!e) return efail(nullptr, GT_ERR_NOMEM, "gt_ens_create: out of host memory");
  e->nm = nmembers;
  e->params.assign(members, members + nmembers);
  e->keys.assign(keys, keys + nmembers);
  const int rko0 = members[0].rko == 4 ? 4 : 2;
  for (int m = 0; m < nmembers; ++m) {
    if (!valid_ens_n(members[m].n) || (members[m].ny != 0 && members[m].ny != members[m].n)) {
      delete e;
      return efail(nullptr, GT_ERR_ARG,
                   "gt_ens_create: member grids must be square, sizes powers of two in [128, 2048]");
    }
    if ((members[m].rko == 4 ? 4 : 2) != rko0) {
      delete e;
      return efail(nullptr, GT_ERR_ARG, "gt_ens_create: all members must use the same RK order");
    }
  }
  e->rko = rko0;
  e->stages = rko0 == 4 ? 4 : 2;
  // one handle per distinct parameter set (members with equal parameters share tables)
  for (int m = 0; m < nmembers; ++m) {
    int found = -1;
    for (size_t q = 0; q < e->handles.size(); ++q)
      if (!std::memcmp(gt::handle_params(e->handles[q]), &members[m], sizeof(gt_params))) found = (int)q;
    if (found < 0) {
      gt_handle* h = nullptr;
      const int rc = gt_create(&members[m], &h);
      if (rc) {
        std::string msg = std::string("gt_ens_create: member ") + std::to_string(m) + ": " + gt_last_error(nullptr);
        free_ens(e);
        delete e;
        return efail(nullptr, rc, msg);
      }
      e->handles.push_back(h);
      found = (int)e->handles.size() - 1;
    }
    e->hidx.push_back(found);
  }
  // work lists, largest members first (their tiles are the longest)
  std::vector<int> order(nmembers);
  for (int m = 0; m < nmembers; ++m) order[m] = m;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return members[a].n > members[b].n; });
  std::vector<EnsTile> col, row;
  std::vector<int2> modes;
  for (int m : order) {
    for (int t = 0; t < gt::ens_col_tiles(members[m].n); ++t) col.push_back({m, t});
    for (int t = 0; t < gt::ens_row_tiles(members[m].n); ++t) row.push_back({m, t});
  }
  for (int m = 0; m < nmembers; ++m) {
    const gt::ForcingView f = gt::handle_forcing(e->handles[e->hidx[m]]);
    for (int k = 0; k < f.nf; ++k) modes.push_back(make_int2(m, k));
  }
  e->ncol = (int)col.size();
  e->nrow = (int)row.size();
  e->nmodes = (int)modes.size();
  cudaError_t c = cudaSuccess;
  auto up = [&](void** dst, const void* src, size_t bytes) {
    if (c != cudaSuccess) return;
    c = cudaMalloc(dst, bytes ? bytes : 8);
    if (c == cudaSuccess && src && bytes) c = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    if (c == cudaSuccess && !src) c = cudaMemset(*dst, 0, bytes ? bytes : 8);
  };
  up((void**)&e->d_col, col.data(), sizeof(EnsTile) * col.size());
  up((void**)&e->d_row, row.data(), sizeof(EnsTile) * row.size());
  up((void**)&e->d_modes, modes.data(), sizeof(int2) * modes.size());
  up((void**)&e->d_flags, nullptr, sizeof(int) * 2 * nmembers);  // even / odd stages
  up((void**)&e->d_args, nullptr, sizeof(NltArgs) * (size_t)e->stages * nmembers);
  up((void**)&e->d_fm, nullptr, sizeof(ForceMember) * nmembers);
  up((void**)&e->d_step, nullptr, sizeof(uint64_t));
  up((void**)&e->d_done, nullptr, sizeof(unsigned));
  if (c == cudaSuccess) c = gt::ens_prepare_r16();
  if (c == cudaSuccess) c = gt::ens_prepare_r8();
  if (c == cudaSuccess) c = gt::ens_prepare_r4();
  if (c == cudaSuccess) c = cudaStreamCreateWithFlags(&e->own, cudaStreamNonBlocking);
  if (c == cudaSuccess) c = cudaEventCreateWithFlags(&e->ev_in, cudaEventDisableTiming);
  if (c == cudaSuccess) c = cudaEventCreateWithFlags(&e->ev_out, cudaEventDisableTiming);
  if (c != cudaSuccess) {
    std::string msg = std::string("gt_ens_create: ") + cudaGetErrorString(c);
    free_ens(e);
    delete e;
    return efail(nullptr, GT_ERR_CUDA, msg);
  }
  *out = e;
  return GT_OK;
}

int gt_ens_destroy(gt_ens* e) {
  if (!e) return GT_OK;
  cudaDeviceSynchronize();
  free_ens(e);
  delete e;
  return GT_OK;
}

const char* gt_ens_last_error(const gt_ens* e) { return e ? e->err.c_str() : gt_last_error(nullptr); }

int gt_ens_set_stream(gt_ens* e, void* stream) {
  if (!e) return efail(nullptr, GT_ERR_ARG, "gt_ens_set_stream: null ensemble");
  e->user = (cudaStream_t)stream;
  return GT_OK;
}

int gt_ens_use_graph(gt_ens* e, int enable) {
  if (!e) return efail(nullptr, GT_ERR_ARG, "gt_ens_use_graph: null ensemble");
  e->use_graph = enable != 0;
  return GT_OK;
}

int gt_ens_set_fields(gt_ens* e, double* const* z, double* const* znl, double* const* znew,
                      double* const* u, double* const* v) {
  if (!e || !z || !znl || !u || !v || (e->rko == 4 && !znew))
    return efail(e, GT_ERR_ARG, "gt_ens_set_fields: null argument");
  const int nm = e->nm;
  e->z.assign(z, z + nm);
  e->znl.assign(znl, znl + nm);
  e->u.assign(u, u + nm);
  e->v.assign(v, v + nm);
  e->znew.assign(nm, nullptr);
  if (znew) e->znew.assign(znew, znew + nm);
  std::vector<NltArgs> args((size_t)e->stages * nm);
  std::vector<ForceMember> fm(nm);
  for (int m = 0; m < nm; ++m) {
    if (!z[m] || !znl[m] || !u[m] || !v[m] || (e->rko == 4 && !znew[m]))
      return efail(e, GT_ERR_ARG, "gt_ens_set_fields: null field pointer");
    gt_handle* h = e->handles[e->hidx[m]];
    // the stage sequence of gt_step_rk2 / gt_step_rk4 (rkstep.f90:2-131); even and odd stages
    // use different flags because pass C of one runs with pass A of the next
    for (int st = 0; st < e->stages; ++st) {
      const double* zin = st == 0 ? z[m] : znl[m];
      int* flag = e->d_flags + (size_t)(st & 1) * nm + m;
      NltArgs a = gt::handle_nlt_args(h, zin, znl[m], u[m], v[m], flag);
      a.epi.z = reinterpret_cast<const double2*>(z[m]);
      a.epi.znew = znew ? reinterpret_cast<double2*>(znew[m]) : nullptr;
      if (e->rko == 4) {
        a.epi.mode = gt::EPI_RK4A + st;
        a.epi.out = reinterpret_cast<double2*>(st == 3 ? z[m] : znl[m]);
      } else {
        a.epi.mode = st == 0 ? gt::EPI_RK2A : gt::EPI_RK2B;
        a.epi.out = reinterpret_cast<double2*>(st == 0 ? znl[m] : z[m]);
      }
      args[(size_t)st * nm + m] = a;
    }
    const gt::ForcingView f = gt::handle_forcing(h);
    fm[m] = ForceMember{reinterpret_cast<double2*>(z[m]), f.ikx, f.iky, f.jc, f.nf, f.nh, f.sf, e->keys[m]};
  }
  GE_CUDA(e, cudaMemcpy(e->d_args, args.data(), sizeof(NltArgs) * args.size(), cudaMemcpyHostToDevice));
  GE_CUDA(e, cudaMemcpy(e->d_fm, fm.data(), sizeof(ForceMember) * fm.size(), cudaMemcpyHostToDevice));
  drop_graph(e);
  e->fields_set = true;
  return GT_OK;
}

int gt_ens_set_step(gt_ens* e, uint64_t step) {
  if (!e) return efail(nullptr, GT_ERR_ARG, "gt_ens_set_step: null ensemble");
  GE_CUDA(e, cudaStreamSynchronize(e->own));
  GE_CUDA(e, cudaMemcpy(e->d_step, &step, sizeof(step), cudaMemcpyHostToDevice));
  return GT_OK;
}

int gt_ens_get_step(gt_ens* e, uint64_t* step) {
  if (!e || !step) return efail(e, GT_ERR_ARG, "gt_ens_get_step: null argument");
  GE_CUDA(e, cudaStreamSynchronize(e->own));
  GE_CUDA(e, cudaMemcpy(step, e->d_step, sizeof(uint64_t), cudaMemcpyDeviceToHost));
  return GT_OK;
}

int gt_ens_step(gt_ens* e, int32_t nsteps) {
  if (!e) return efail(nullptr, GT_ERR_ARG, "gt_ens_step: null ensemble");
  if (!e->fields_set) return efail(e, GT_ERR_STATE, "gt_ens_step: call gt_ens_set_fields first");
  if (nsteps <= 0) return GT_OK;
  GE_CUDA(e, cudaEventRecord(e->ev_in, e->user));
  GE_CUDA(e, cudaStreamWaitEvent(e->own, e->ev_in, 0));
  if (e->use_graph) {
    if (!e->gexec) {
      GE_CUDA(e, cudaStreamBeginCapture(e->own, cudaStreamCaptureModeThreadLocal));
      const int rc = enqueue_step(e, e->own);
      cudaGraph_t g = nullptr;
      const cudaError_t c = cudaStreamEndCapture(e->own, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (c != cudaSuccess) return ecuda(e, c, "cudaStreamEndCapture");
      e->graph = g;
      GE_CUDA(e, cudaGraphInstantiate(&e->gexec, e->graph, 0));
    }
    for (int s = 0; s < nsteps; ++s) GE_CUDA(e, cudaGraphLaunch(e->gexec, e->own));
  } else {
    for (int s = 0; s < nsteps; ++s) {
      const int rc = enqueue_step(e, e->own);
      if (rc) return rc;
    }
  }
  GE_CUDA(e, cudaEventRecord(e->ev_out, e->own));
  GE_CUDA(e, cudaStreamWaitEvent(e->user, e->ev_out, 0));
  return GT_OK;
}

int gt_ens_set_tile(gt_ens* e, int32_t values_per_thread) {
  if (!e) return efail(nullptr, GT_ERR_ARG, "gt_ens_set_tile: null ensemble");
  if (values_per_thread != 16 && values_per_thread != 8 && values_per_thread != 4)
    return efail(e, GT_ERR_ARG, "gt_ens_set_tile: values per thread must be 16, 8 or 4");
  if (values_per_thread != e->tile_r) {
    GE_CUDA(e, cudaStreamSynchronize(e->own));
    drop_graph(e);  // the next step captures the new family
    e->tile_r = values_per_thread;
  }
  return GT_OK;
}

int gt_ens_get_tile(const gt_ens* e, int32_t* values_per_thread) {
  if (!e || !values_per_thread) return efail(nullptr, GT_ERR_ARG, "gt_ens_get_tile: null argument");
  *values_per_thread = e->tile_r;
  return GT_OK;
}

int gt_ens_autotune(gt_ens* e, int32_t steps, double* ms_per_step, int32_t* best) {
  if (!e) return efail(nullptr, GT_ERR_ARG, "gt_ens_autotune: null ensemble");
  if (!e->fields_set) return efail(e, GT_ERR_STATE, "gt_ens_autotune: call gt_ens_set_fields first");
  if (steps < 1) return efail(e, GT_ERR_ARG, "gt_ens_autotune: steps must be >= 1");
  static const int fam[3] = {16, 8, 4};
  // the members' fields and the step counter are put back afterwards
  std::vector<size_t> off(e->nm + 1, 0);
  for (int m = 0; m < e->nm; ++m) {
    const int n = e->params[m].n;
    off[m + 1] = off[m] + sizeof(double) * (size_t)(n + 2) * n;
  }
  char* backup = nullptr;
  GE_CUDA(e, cudaStreamSynchronize(e->user));
  GE_CUDA(e, cudaMalloc((void**)&backup, off[e->nm]));
  uint64_t step0 = 0;
  int rc = GT_OK;
  cudaError_t c = cudaMemcpy(&step0, e->d_step, sizeof(step0), cudaMemcpyDeviceToHost);
  for (int m = 0; m < e->nm && c == cudaSuccess; ++m)
    c = cudaMemcpy(backup + off[m], e->z[m], off[m + 1] - off[m], cudaMemcpyDeviceToDevice);
  cudaEvent_t ev[2] = {nullptr, nullptr};
  if (c == cudaSuccess) c = cudaEventCreate(&ev[0]);
  if (c == cudaSuccess) c = cudaEventCreate(&ev[1]);
  if (c != cudaSuccess) rc = ecuda(e, c, "gt_ens_autotune: set-up");
  const int saved = e->tile_r;
  double ms[3] = {-1.0, -1.0, -1.0};
  int bi = -1;
  for (int q = 0; q < 3 && !rc; ++q) {
    rc = gt_ens_set_tile(e, fam[q]);
    if (!rc) rc = gt_ens_step(e, 2);  // capture + warm-up
    if (!rc) c = cudaEventRecord(ev[0], e->user);
    if (!rc && c == cudaSuccess) rc = gt_ens_step(e, steps);
    if (!rc && c == cudaSuccess) c = cudaEventRecord(ev[1], e->user);
    if (!rc && c == cudaSuccess) c = cudaEventSynchronize(ev[1]);
    float t = 0.0f;
    if (!rc && c == cudaSuccess) c = cudaEventElapsedTime(&t, ev[0], ev[1]);
    if (!rc && c != cudaSuccess) rc = ecuda(e, c, "gt_ens_autotune: timing");
    if (!rc) {
      ms[q] = (double)t / steps;
      if (bi < 0 || ms[q] < ms[bi]) bi = q;
    }
  }
  // restore the fields and the step counter whatever happened
  cudaStreamSynchronize(e->own);
  for (int m = 0; m < e->nm; ++m)
    cudaMemcpy(e->z[m], backup + off[m], off[m + 1] - off[m], cudaMemcpyDeviceToDevice);
  cudaMemcpy(e->d_step, &step0, sizeof(step0), cudaMemcpyHostToDevice);
  cudaFree(backup);
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  const int keep = rc ? saved : fam[bi];
  const int rc2 = gt_ens_set_tile(e, keep);
  if (rc) return rc;
  if (rc2) return rc2;
  if (ms_per_step)
    for (int q = 0; q < 3; ++q) ms_per_step[q] = ms[q];
  if (best) *best = keep;
  return GT_OK;
}

int gt_forcing_philox(gt_handle* h, double* z, uint64_t key, uint64_t step) {
  if (!h || !z) return gt::set_error(h, GT_ERR_ARG, "gt_forcing_philox: null argument");
  const gt::ForcingView f = gt::handle_forcing(h);
  if (f.nf == 0) return GT_OK;
  ForceMember m{reinterpret_cast<double2*>(z), f.ikx, f.iky, f.jc, f.nf, f.nh, f.sf, key};
  gt::k_forcing_philox1<<<(f.nf + 127) / 128, 128, 0, gt::handle_stream(h)>>>(m, step);
  const cudaError_t c = cudaGetLastError();
  if (c != cudaSuccess) return gt::set_error(h, GT_ERR_CUDA, cudaGetErrorString(c));
  return GT_OK;
}

}  // extern "C"
