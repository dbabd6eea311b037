// gturbo.cu -- host side of the C-ABI declared in include/gturbo.h.
//
// A handle owns the tables of one parameter set (defk + iniforcing of the reference, the
// twiddles, the truncation cut-offs and the LCG jump-ahead coefficients) on the device that
// was current at gt_create. Fields are owned by the caller and passed as device pointers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/gturbo.h"
#include "gt_misc.cuh"
#include "gt_ops.h"
#include "gt_internal.h"

using gt::GtOp;

namespace {

thread_local std::string g_create_error;

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

struct gt_handle {
  gt_params p;
  // N = NX (row length, x fastest), NY rows, NH = NX/2+1 columns of the spectral field
  int N = 0, NY = 0, NH = 0, NBIN = 0, split = 0, rko = 2, truncate = 1;
  bool rt = false;  // non-square: column kernels with the column count at run time (variants 1, 2)
  int kxlim = 0;
  double dkx = 0, dky = 0, dt2 = 0, dt3 = 0, dt6 = 0, sdt = 0;
  double fkxsmax = 0, fkysmax = 0, rtrunc2 = 0;
  int nf = 0;
  double inpz = 0, inpe = 0;
  std::vector<double> fkx, fky, fkxs, fkys, emkx, emky;
  std::vector<int> jc, kcut, ikxf, ikyf;
  std::vector<uint32_t> lcga, lcgb;  // index k: coefficients of the (k+1)-th draw
  uint32_t lcga_nf = 1, lcgb_nf = 0;
  // forced-mode map of the fused kick (EpiArgs::fmap); fuse_ok = 0 when two kicks would land
  // on one value (a self-conjugate mode), which keeps the separate forcing launch
  std::vector<int> fmap;
  int fwi = 0, fwj = 0, fh = 0, fuse_ok = 0;
  // the step's kick increments, computed on a side stream while the step's first passes run
  double2* d_kick = nullptr;
  cudaStream_t kick_stream = nullptr;
  cudaEvent_t kick_fork = nullptr, kick_join = nullptr;
  int device = 0;
  int variant = 0;      // launch variant of the column passes
  int row_variant = 0;  // launch variant of the row passes
  cudaStream_t stream = nullptr;
  std::string err;
  // device tables
  double2* d_tw = nullptr;   // column transforms (length NY)
  double2* d_twr = nullptr;  // row transforms (length NX); null for a square grid (d_tw serves)
  double* d_emk = nullptr;
  double* d_kainv = nullptr;
  double *d_fkx = nullptr, *d_fky = nullptr, *d_fkxs = nullptr, *d_fkys = nullptr;
  double *d_emkx = nullptr, *d_emky = nullptr;
  int *d_kcut = nullptr, *d_jc = nullptr, *d_ikxf = nullptr, *d_ikyf = nullptr, *d_fmap = nullptr;
  uint32_t *d_lcga = nullptr, *d_lcgb = nullptr;
  double2* d_ff = nullptr;
  int* d_flag = nullptr;
  // field-split column passes (N <= 2048): q goes to the handle's own field; in mode 1 pass C's
  // two CTAs per column meet at a per-column counter (mode 2 forms 2-CTA clusters instead), as
  // do the transposed and tangent pass C's CTAs
  double2* d_qscr = nullptr;
  int* d_colcnt = nullptr;
  int col_split = 2;  // use them where the column variant allows (gt_set_col_split: 0, 1, 2)
  int pdl = 1;        // programmatic dependent launch of the pass kernels (gt_set_pdl)
  int64_t adj_mem = 0;  // device memory for whole kept segments of gt_adj_gradient (gt_adj_set_memory)
  // CUDA graphs of the steps (gt_set_graphs): a few captured steps, keyed by kind, fields and
  // launch settings; the fused kick's LCG state is the only parameter that changes between calls
  struct StepGraph {
    int kind = 0;
    const void* f[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    int variant = 0, row_variant = 0, col_split = 0, pdl = 0;
    cudaGraph_t graph = nullptr;     // kept alive: its node handles address the instance
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t kick = nullptr;  // the k_kick_values node of a forced step
    unsigned long long used = 0;
  };
  int graphs = 1;
  bool graph_failed = false;  // a capture failed once, or captures kept evicting one another
  unsigned long long sg_captures = 0, sg_replays = 0;
  std::vector<StepGraph> sg;
  unsigned long long sg_clock = 0;
  cudaStream_t cap_stream = nullptr;
  // diagnostics scratch
  double *d_part = nullptr, *d_rowsum = nullptr, *d_bins = nullptr, *d_fl = nullptr, *d_glob = nullptr;
  double* h_diag = nullptr;  // pinned: bins [nbin*4] + fl [nbin*2] + glob [6]
  cudaError_t (*dispatch)(const GtOp&) = nullptr;      // column passes: the NY instantiation
  cudaError_t (*dispatch_row)(const GtOp&) = nullptr;  // row passes: the NX instantiation
  // launch timing (gt_profile)
  bool prof = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_kind;  // kind of pair p = events 2p, 2p+1
};

namespace gt {

NltArgs handle_nlt_args(const gt_handle* h, const double* zin, double* q, double* u, double* v,
                        int* flag) {
  NltArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n = h->N;
  a.zin = reinterpret_cast<const double2*>(zin);
  a.q = reinterpret_cast<double2*>(q);
  a.u = reinterpret_cast<double2*>(u);
  a.v = reinterpret_cast<double2*>(v);
  a.kainv = h->d_kainv;
  a.fkx = h->d_fkx;
  a.fky = h->d_fky;
  a.kcut = h->d_kcut;
  a.tw = h->d_tw;
  a.twr = h->d_twr ? h->d_twr : h->d_tw;
  a.nh = h->NH;
  a.cscale = 0.5 / ((double)h->N * (double)h->NY);
  a.truncate = h->truncate;
  a.kxlim = h->truncate ? h->kxlim : h->N / 2;
  a.kin = a.kxlim;
  a.kout = a.kxlim;
  a.flag = flag;
  a.colcnt = h->d_colcnt;
  a.epi.split = h->split;
  a.epi.emk = h->d_emk;
  a.epi.emkx = h->d_emkx;
  a.epi.emky = h->d_emky;
  a.epi.dt = h->p.dt;
  a.epi.dt2 = h->dt2;
  a.epi.dt3 = h->dt3;
  a.epi.dt6 = h->dt6;
  a.epi.ny = h->NY;
  return a;
}

ForcingView handle_forcing(const gt_handle* h) {
  ForcingView f;
  f.ikx = h->d_ikxf;
  f.iky = h->d_ikyf;
  f.jc = h->d_jc;
  f.nf = h->nf;
  f.nh = h->NH;
  f.sf = h->sdt * h->p.famp;
  f.lcga = h->d_lcga;
  f.lcgb = h->d_lcgb;
  f.lcga_nf = h->lcga_nf;
  f.lcgb_nf = h->lcgb_nf;
  f.sdt = h->sdt;
  return f;
}

cudaError_t handle_dispatch(const gt_handle* h, const GtOp& op) {
  return is_row_op(op.kind) ? h->dispatch_row(op) : h->dispatch(op);
}

cudaError_t forcing_amp(gt_handle* h, double* z, uint32_t seed0, double famp) {
  if (h->nf == 0) return cudaSuccess;
  k_forcing<<<(h->nf + 127) / 128, 128, 0, h->stream>>>(
      reinterpret_cast<double2*>(z), h->NH, h->nf, h->d_ikxf, h->d_ikyf, h->d_jc, h->d_lcga,
      h->d_lcgb, h->d_ff, seed0, h->sdt * famp);
  return cudaGetLastError();
}

void handle_k2(const gt_handle* h, const double** fkxs, const double** fkys) {
  *fkxs = h->d_fkxs;
  *fkys = h->d_fkys;
}

int* handle_flag(const gt_handle* h) { return h->d_flag; }

const gt_params* handle_params(const gt_handle* h) { return &h->p; }
int handle_rko(const gt_handle* h) { return h->rko; }
int handle_variant(const gt_handle* h) { return h->variant; }
int handle_row_variant(const gt_handle* h) { return h->row_variant; }
cudaStream_t handle_stream(const gt_handle* h) { return h->stream; }

}  // namespace gt

namespace {

int fail(gt_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  else g_create_error = msg;
  return code;
}

}  // namespace

int gt::set_error(gt_handle* h, int code, const char* msg) { return fail(h, code, msg); }

namespace {

int cuda_fail(gt_handle* h, cudaError_t e, const char* what) {
  return fail(h, GT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define GT_CUDA(h, call)                                   \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

bool pow2_in_range(int n) { return n >= 16 && n <= 8192 && (n & (n - 1)) == 0; }

// A grid NX x NY: both powers of two in [16, 8192]; a non-square grid has both sides >= 32, so
// that its row count is a multiple of every row pass's rows per CTA (at most 32).
// Its columns (length NY) run the column variants 1 or 2, so NY <= 4096.
bool grid_ok(int nx, int ny) {
  return pow2_in_range(nx) && pow2_in_range(ny) && (nx == ny || (nx >= 32 && ny >= 32 && ny <= 4096));
}

// Column variant v exists for the handle's grid: for its column length, and, on a non-square grid,
// among the variants whose column kernels take the column count at run time (1 and 2).
bool col_variant_ok(const gt_handle* h, int v) {
  return gt_variant_supported(h->NY, v) && (!h->rt || v == 1 || v == 2);
}

// The row variant that goes with column variant v in gt_set_variant: the same launch variant.
int natural_row_variant(int v) { return v; }

// The twiddle buffer of the FFT passes (gt_fft.cuh): exp(-2 pi i k / n) for k in [0, n), each
// value from an argument reduced to [0, pi/4]; then the Linzer-Feig forms tw[n + k] = (c, t) with
// tw[k] = c (1 + i t); then the radix-16, 8 and 4 pass tables built from those (make_lf_entry),
// one per pass span, field by field (lf_pass_table).
// c = Re tw[k], except at k = n/4 and 3n/4 (Re tw[k] = 0), where c = 2^-60 and
// t = Im tw[k] / c = -+2^60: c t is exact and Re(c (1 + i t)) = 2^-60 is far below the rounding
// of the other entries.
void make_twiddles(int n, std::vector<double2>& tw) {
  tw.assign((size_t)gt::twiddle_buffer_size(n), make_double2(0.0, 0.0));
  const double twopi = 2.0 * 3.14159265358979323846;
  const int q4 = n / 4;
  for (int k = 0; k < n; ++k) {
    const int quad = k / q4, r = k % q4;
    double c, s;
    if (2 * r <= q4) {
      c = std::cos(twopi * (double)r / (double)n);
      s = std::sin(twopi * (double)r / (double)n);
    } else {
      c = std::sin(twopi * (double)(q4 - r) / (double)n);
      s = std::cos(twopi * (double)(q4 - r) / (double)n);
    }
    double C, S;
    switch (quad) {
      case 0: C = c; S = s; break;
      case 1: C = -s; S = c; break;
      case 2: C = -c; S = -s; break;
      default: C = s; S = -c; break;
    }
    tw[k] = make_double2(C, -S);
  }
  for (int k = 0; k < n; ++k) {
    const double c = tw[k].x != 0.0 ? tw[k].x : std::ldexp(1.0, -60);
    tw[n + k] = make_double2(c, tw[k].y / c);
  }
  const double2* lf = tw.data() + n;
  auto fill = [&](auto rp_tag) {
    constexpr int RP = decltype(rp_tag)::value;
    constexpr int E = gt::lf_entry_doubles(RP);
    double e[E];
    for (int ns = 2; ns <= n / RP; ns *= 2) {
      double2* tab = tw.data() + gt::lf_pass_table(RP, n, ns);
      for (int k = 0; k < ns; ++k) {
        gt::make_lf_entry<RP>(lf, n, k * (n / (ns * RP)), e);
        for (int q = 0; q < E / 2; ++q) tab[(size_t)q * ns + k] = make_double2(e[2 * q], e[2 * q + 1]);
      }
    }
  };
  fill(std::integral_constant<int, 16>());
  fill(std::integral_constant<int, 8>());
  fill(std::integral_constant<int, 4>());
}

template <typename T>
int upload(gt_handle* h, T** dst, const T* src, size_t count) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)dst, sizeof(T) * count);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMalloc");
  if (src) {
    e = cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemcpy");
  }
  return GT_OK;
}

cudaError_t (*dispatch_for(int n))(const GtOp&) {
  switch (n) {
    case 16: return gt::dispatch_16;
    case 32: return gt::dispatch_32;
    case 64: return gt::dispatch_64;
    case 128: return gt::dispatch_128;
    case 256: return gt::dispatch_256;
    case 512: return gt::dispatch_512;
    case 1024: return gt::dispatch_1024;
    case 2048: return gt::dispatch_2048;
    case 4096: return gt::dispatch_4096;
    case 8192: return gt::dispatch_8192;
    default: return nullptr;
  }
}

cudaError_t prepare_for(int n) {
  switch (n) {
    case 16: return gt::prepare_16();
    case 32: return gt::prepare_32();
    case 64: return gt::prepare_64();
    case 128: return gt::prepare_128();
    case 256: return gt::prepare_256();
    case 512: return gt::prepare_512();
    case 1024: return gt::prepare_1024();
    case 2048: return gt::prepare_2048();
    case 4096: return gt::prepare_4096();
    case 8192: return gt::prepare_8192();
    default: return cudaErrorInvalidValue;
  }
}

void free_device(gt_handle* h) {
  void* ptrs[] = {h->d_tw, h->d_twr, h->d_emk, h->d_kainv, h->d_fkx, h->d_fky, h->d_fkxs, h->d_fkys,
                  h->d_emkx, h->d_emky, h->d_kcut, h->d_jc, h->d_ikxf, h->d_ikyf, h->d_lcga,
                  h->d_lcgb, h->d_ff, h->d_flag, h->d_part, h->d_rowsum, h->d_bins, h->d_fl,
                  h->d_glob, h->d_fmap, h->d_qscr, h->d_colcnt, h->d_kick};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (h->h_diag) cudaFreeHost(h->h_diag);
}

GtOp base_op(const gt_handle* h) {
  GtOp op;
  std::memset(&op, 0, sizeof(op));
  op.stream = h->stream;
  op.variant = h->variant;
  op.row_variant = h->row_variant;
  op.tw = h->d_tw;
  op.twr = h->d_twr ? h->d_twr : h->d_tw;
  op.nh = h->NH;
  op.nrows = h->NY;
  op.rt = h->rt;
  op.nlt = gt::handle_nlt_args(h, nullptr, nullptr, nullptr, nullptr, h->d_flag);
  op.pdl = gt::handle_pdl(h);
  op.cluster = h->col_split == 2;
  return op;
}

// Event pair around the next launch when profiling: prof_begin before, prof_end after.
int prof_begin(gt_handle* h, int kind) {
  if (!h->prof) return -1;
  const size_t pair = h->ev_kind.size();
  while (h->ev_pool.size() < 2 * (pair + 1)) {
    cudaEvent_t ev;
    if (cudaEventCreate(&ev) != cudaSuccess) return -1;
    h->ev_pool.push_back(ev);
  }
  h->ev_kind.push_back(kind);
  cudaEventRecord(h->ev_pool[2 * pair], h->stream);
  return (int)pair;
}

void prof_end(gt_handle* h, int pair) {
  if (pair >= 0) cudaEventRecord(h->ev_pool[2 * pair + 1], h->stream);
}

int op_class(int kind) {
  switch (kind) {
    case gt::OP_NLT_COLINV: return GT_PROF_NLT_COLINV;
    case gt::OP_NLT_ROW: return GT_PROF_NLT_ROW;
    case gt::OP_NLT_COLFWD: return GT_PROF_NLT_COLFWD;
    case gt::OP_NLT_COLFWD_INV: return GT_PROF_NLT_COLFWD_INV;
    case gt::OP_NLT_COLINV_FS: return GT_PROF_NLT_COLINV;
    case gt::OP_NLT_COLFWD_FS: return GT_PROF_NLT_COLFWD;
    default: return GT_PROF_OTHER;
  }
}

int run(gt_handle* h, const GtOp& op) {
  const int pair = prof_begin(h, op_class(op.kind));
  cudaError_t e = gt::handle_dispatch(h, op);
  prof_end(h, pair);
  if (e != cudaSuccess) return cuda_fail(h, e, "kernel launch");
  return GT_OK;
}

// The field-split column passes run when the handle has their scratch (N <= 2048), the user
// has not turned them off, and the column variant has one column per CTA without thread groups.
bool split_active(const gt_handle* h) {
  const bool one_col =
      (h->variant == 0 && h->NY >= 1024) || h->variant == 1 || h->variant == 2 || h->variant == 5;
  return h->col_split && h->d_qscr && one_col;
}

// One nonlinear-term evaluation: input zin, work fields (qbuf receives the transformed q;
// it may alias zin), u, v; pass C applies the epilogue `epi`. The field-split passes put q in
// the handle's own field instead.
int nlt_passes(gt_handle* h, const double* zin, double* qbuf, double* u, double* v,
               const gt::EpiArgs& epi) {
  GtOp op = base_op(h);
  if (split_active(h)) {
    op.nlt = gt::handle_nlt_args(h, zin, reinterpret_cast<double*>(h->d_qscr), u, v, h->d_flag);
    op.nlt.epi = epi;
    op.kind = gt::OP_NLT_COLINV_FS;
    int rc = run(h, op);
    if (rc) return rc;
    op.kind = gt::OP_NLT_ROW;
    rc = run(h, op);
    if (rc) return rc;
    op.kind = gt::OP_NLT_COLFWD_FS;
    return run(h, op);
  }
  op.nlt = gt::handle_nlt_args(h, zin, qbuf, u, v, h->d_flag);
  op.nlt.epi = epi;
  op.kind = gt::OP_NLT_COLINV;
  int rc = run(h, op);
  if (rc) return rc;
  op.kind = gt::OP_NLT_ROW;
  rc = run(h, op);
  if (rc) return rc;
  op.kind = gt::OP_NLT_COLFWD;
  return run(h, op);
}

gt::EpiArgs make_epi(const gt_handle* h, int mode, double* out, double* znew, const double* z) {
  gt::EpiArgs E = base_op(h).nlt.epi;
  E.mode = mode;
  E.out = reinterpret_cast<double2*>(out);
  E.znew = reinterpret_cast<double2*>(znew);
  E.z = reinterpret_cast<const double2*>(z);
  return E;
}

}  // namespace

namespace gt {
bool handle_col_split(const gt_handle* h) { return split_active(h); }
bool handle_col_cluster(const gt_handle* h) { return h->col_split == 2; }
// the per-launch timing events of the profiling mode sit between the kernels: no overlap there
bool handle_pdl(const gt_handle* h) { return h->pdl && !h->prof; }
int64_t handle_adj_memory(const gt_handle* h) { return h->adj_mem; }
}  // namespace gt

extern "C" {

int gt_create(const gt_params* p, gt_handle** out) {
  if (!p || !out) return fail(nullptr, GT_ERR_ARG, "gt_create: null argument");
  *out = nullptr;
  const int ny_in = p->ny > 0 ? p->ny : p->n;
  if (p->ny < 0 || !grid_ok(p->n, ny_in))
    return fail(nullptr, GT_ERR_ARG,
                "gt_create: n (NX) and ny (NY) must each be a power of two in [16, 8192]; a non-square grid "
                "has both >= 32 and ny <= 4096");
  if (!(p->xlx > 0.0) || !(p->xly > 0.0) || !(p->dt > 0.0))
    return fail(nullptr, GT_ERR_ARG, "gt_create: xlx, xly and dt must be positive");
  gt_handle* h = new (std::nothrow) gt_handle();
  if (!h) return fail(nullptr, GT_ERR_NOMEM, "gt_create: out of host memory");
  h->p = *p;
  h->p.ny = ny_in;
  const int N = h->N = p->n;  // NX
  const int NY = h->NY = ny_in;
  const int NH = h->NH = N / 2 + 1;
  h->NBIN = N / 2;
  h->rt = N != NY;
  h->dispatch = dispatch_for(NY);
  h->dispatch_row = dispatch_for(N);
  // The launch variants that timed fastest on GB300 for this grid size (RK2 and RK4 alike).
  // Columns: grouped with 4 values per thread at 16^2, 2 values per thread from 32^2 to 256^2,
  // 4 at 512^2 and 1024^2, 8 at 2048^2, 16 at 4096^2, 8 at 8192^2. Rows: grouped with 4 values per
  // thread at 16^2, grouped with 2 from 32^2 to 128^2, 4 values per thread at 256^2 and 512^2,
  // 8 at 1024^2 and 2048^2, 16 from 4096^2 up. gt_autotune re-times.
  // (Columns follow the column length NY, rows the row length NX.)
  h->variant = NY < 32 ? 3 : NY <= 256 ? 5 : NY <= 1024 ? 2 : (NY == 2048 || NY == 8192) ? 1 : 0;
  if (h->rt) h->variant = NY <= 1024 ? 2 : 1;
  h->row_variant = N < 32 ? 3 : N <= 128 ? 5 : N <= 512 ? 2 : N <= 2048 ? 1 : 0;
  // inieuler.f90:22-36, 237-244
  int split = 0;
  if (p->alpnu < 1.0005 && p->alpnu > 0.9995 && p->alpmu < 0.0005 && p->alpmu > -0.0005) split = 1;
  if (p->rko == 4) split = 0;
  if (p->split == 0 || p->split == 1) split = p->split;
  h->split = split;
  h->rko = (p->rko == 4) ? 4 : 2;
  if (h->split && h->rko == 4) {
    delete h;
    return fail(nullptr, GT_ERR_ARG, "gt_create: the split integrator exists only for RK2");
  }
  h->truncate = p->truncate;
  // inieuler.f90:78-81
  h->sdt = std::sqrt(p->dt);
  h->dt2 = p->dt / 2.0;
  h->dt3 = p->dt / 3.0;
  h->dt6 = p->dt / 6.0;
  // defk.f90:12-73 (x over NX/2+1 columns, y over NY rows)
  h->jc.resize(NY);
  h->jc[0] = 0;
  for (int j = 1; j < NY; ++j) h->jc[j] = NY - j;
  h->dkx = 2.0 * 3.14159265358979323846 / p->xlx;
  h->dky = 2.0 * 3.14159265358979323846 / p->xly;
  h->fkx.resize(NH);
  h->fkxs.resize(NH);
  h->fky.resize(NY);
  h->fkys.resize(NY);
  for (int i = 0; i < NH; ++i) h->fkx[i] = (double)i * h->dkx;
  for (int j = 0; j <= NY / 2; ++j) h->fky[j] = (double)j * h->dky;
  for (int j = NY / 2 + 1; j < NY; ++j) h->fky[j] = (double)(j - NY) * h->dky;
  for (int i = 0; i < NH; ++i) h->fkxs[i] = h->fkx[i] * h->fkx[i];
  for (int j = 0; j < NY; ++j) h->fkys[j] = h->fky[j] * h->fky[j];
  h->emky.resize(NY);
  h->emkx.resize(NH);
  for (int j = 0; j < NY; ++j)
    h->emky[j] = std::exp(-0.5 * p->dt * (p->nu * std::pow(h->fkys[j], p->alpnu) + p->mu));
  for (int i = 0; i < NH; ++i)
    h->emkx[i] = std::exp(-0.5 * p->dt * (p->nu * std::pow(h->fkxs[i], p->alpnu)));
  h->fkxsmax = h->fkxs[N / 2];
  h->fkysmax = h->fkys[NY / 2];
  h->rtrunc2 = p->rtrunc * p->rtrunc;
  // truncation cut-off per column: largest |ky| row kept by trunc.f90:12-16 (monotone in |ky|)
  h->kcut.resize(NH);
  h->kxlim = -1;
  for (int i = 0; i < NH; ++i) {
    int a = 0;
    while (a <= NY / 2) {
      const double k1 = h->fkys[a] / h->fkysmax;
      const double k2 = k1 + h->fkxs[i] / h->fkxsmax;
      if (k2 > h->rtrunc2) break;
      ++a;
    }
    h->kcut[i] = a - 1;
    if (a > 0) h->kxlim = i;
  }
  // iniforcing.f90:11-68
  const double famp = p->famp, k1f2 = p->k1f * p->k1f, k2f2 = p->k2f * p->k2f;
  for (int pass = 0; pass < 3; ++pass) {
    const int ilo = pass == 0 ? 0 : pass == 1 ? 1 : N / 2;
    const int ihi = pass == 0 ? 0 : pass == 1 ? N / 2 - 1 : N / 2;
    for (int i = ilo; i <= ihi; ++i) {
      const int jlo = pass == 0 ? 1 : 0;
      const int jhi = pass == 1 ? NY - 1 : NY / 2;
      for (int j = jlo; j <= jhi; ++j) {
        const double k2 = h->fkxs[i] + h->fkys[j];
        const double k2n = h->fkxs[i] / h->fkxsmax + h->fkys[j] / h->fkysmax;
        if (k2n <= h->rtrunc2 && k2 <= k2f2 && k2 > k1f2) {
          if ((int)h->ikxf.size() >= GT_NFORC) {
            delete h;
            return fail(nullptr, GT_ERR_NFORC, "NFORC too small !");
          }
          h->ikxf.push_back(i);
          h->ikyf.push_back(j);
          h->inpz = h->inpz + famp * famp;
          h->inpe = h->inpe + famp * famp / std::pow(k2, p->alpv / 2.0);
        }
      }
    }
  }
  h->nf = (int)h->ikxf.size();
  // LCG jump-ahead: x_{k+1} = A_{k+1} x_0 + B_{k+1} (mod 2^32, masked to 31 bits)
  uint32_t A = 1, B = 0;
  for (int k = 0; k < h->nf; ++k) {
    A = 69069u * A;
    B = 69069u * B + 1u;
    h->lcga.push_back(A);
    h->lcgb.push_back(B);
  }
  h->lcga_nf = A;
  h->lcgb_nf = B;
  // map of the forced values for the fused kick: mode k at (ikx, iky), and its conjugate partner
  // (ikx, jc[iky]) on the kx = 0 and Nyquist columns (forcing.f90:21-31)
  if (h->nf > 0) {
    auto aky = [&](int j) { return j <= NY / 2 ? j : NY - j; };
    for (int k = 0; k < h->nf; ++k) {
      h->fwi = std::max(h->fwi, h->ikxf[k] + 1);
      h->fwj = std::max(h->fwj, aky(h->ikyf[k]) + 1);
    }
    h->fh = std::min(NY, 2 * h->fwj - 1);
    h->fmap.assign((size_t)h->fwi * h->fh, -1);
    h->fuse_ok = 1;
    auto put = [&](int i, int j, int e) {
      const int jj = j < h->fwj ? j : j - (NY - h->fh);
      int& slot = h->fmap[(size_t)i * h->fh + jj];
      if (slot >= 0) h->fuse_ok = 0;
      slot = e;
    };
    for (int k = 0; k < h->nf; ++k) {
      const int i = h->ikxf[k], j = h->ikyf[k];
      put(i, j, k);
      if (i == 0 || i == NH - 1) put(i, h->jc[j], k | (1 << 30));
    }
  }

  // device side
  int rc = GT_OK;
  cudaError_t e = cudaGetDevice(&h->device);
  if (e != cudaSuccess) rc = cuda_fail(h, e, "cudaGetDevice");
  if (!rc) {
    e = prepare_for(NY);
    if (e == cudaSuccess && NY != N) e = prepare_for(N);
    if (e == cudaSuccess && std::max(N, NY) >= 4096) e = gt::diag_prepare();
    if (e != cudaSuccess) rc = cuda_fail(h, e, "cudaFuncSetAttribute");
  }
  std::vector<double2> tw, twr;
  make_twiddles(NY, tw);
  if (NY != N) make_twiddles(N, twr);
  std::vector<double2> ff(h->nf > 0 ? h->nf : 1, make_double2(1.0, 1.0));
  const size_t nc = (size_t)NY * NH;
  if (!rc) rc = upload(h, &h->d_tw, tw.data(), tw.size());
  if (!rc && NY != N) rc = upload(h, &h->d_twr, twr.data(), twr.size());
  if (!rc) rc = upload<double>(h, &h->d_emk, nullptr, nc);
  if (!rc) rc = upload<double>(h, &h->d_kainv, nullptr, nc);
  if (!rc) rc = upload(h, &h->d_fkx, h->fkx.data(), NH);
  if (!rc) rc = upload(h, &h->d_fky, h->fky.data(), NY);
  if (!rc) rc = upload(h, &h->d_fkxs, h->fkxs.data(), NH);
  if (!rc) rc = upload(h, &h->d_fkys, h->fkys.data(), NY);
  if (!rc) rc = upload(h, &h->d_emkx, h->emkx.data(), NH);
  if (!rc) rc = upload(h, &h->d_emky, h->emky.data(), NY);
  if (!rc) rc = upload(h, &h->d_kcut, h->kcut.data(), NH);
  if (!rc) rc = upload(h, &h->d_jc, h->jc.data(), NY);
  if (!rc) rc = upload(h, &h->d_ikxf, h->ikxf.data(), h->nf);
  if (!rc) rc = upload(h, &h->d_ikyf, h->ikyf.data(), h->nf);
  if (!rc) rc = upload(h, &h->d_lcga, h->lcga.data(), h->nf);
  if (!rc) rc = upload(h, &h->d_lcgb, h->lcgb.data(), h->nf);
  if (!rc) rc = upload(h, &h->d_ff, ff.data(), ff.size());
  if (!rc && h->nf > 0) rc = upload(h, &h->d_fmap, h->fmap.data(), h->fmap.size());
  if (!rc && h->nf > 0) rc = upload<double2>(h, &h->d_kick, nullptr, (size_t)h->nf);
  if (!rc && NY <= 2048) {  // the field-split column passes (column length up to 2048)
    const std::vector<int> zeros(NH, 0);
    rc = upload<double2>(h, &h->d_qscr, nullptr, (size_t)NY * NH);
    if (!rc) rc = upload(h, &h->d_colcnt, zeros.data(), NH);
  }
  const int zeros2[2] = {0, 0};  // untruncated-input flags of even / odd stages
  if (!rc) rc = upload(h, &h->d_flag, zeros2, 2);
  const int ngroups = gt::diag_groups(NY);
  if (!rc) rc = upload<double>(h, &h->d_part, nullptr, (size_t)ngroups * h->NBIN * 4);
  if (!rc) rc = upload<double>(h, &h->d_rowsum, nullptr, (size_t)NY * 6);
  if (!rc) rc = upload<double>(h, &h->d_bins, nullptr, (size_t)h->NBIN * 4);
  if (!rc) rc = upload<double>(h, &h->d_fl, nullptr, (size_t)h->NBIN * 2);
  if (!rc) rc = upload<double>(h, &h->d_glob, nullptr, 6);
  if (!rc) {
    e = cudaMallocHost((void**)&h->h_diag, sizeof(double) * ((size_t)h->NBIN * 6 + 6));
    if (e != cudaSuccess) rc = cuda_fail(h, e, "cudaMallocHost");
  }
  if (!rc) {
    gt::k_init_tables<<<1024, 256>>>(h->d_emk, h->d_kainv, h->d_fkxs, h->d_fkys, NY, NH, p->nu,
                                      p->alpnu, p->mu, p->alpmu, p->alpv, p->dt);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) rc = cuda_fail(h, e, "table set-up");
  }
  if (rc) {
    g_create_error = h->err;
    free_device(h);
    delete h;
    return rc;
  }
  *out = h;
  return GT_OK;
}

static void drop_step_graphs(gt_handle* h);

int gt_destroy(gt_handle* h) {
  if (!h) return GT_OK;
  cudaDeviceSynchronize();
  drop_step_graphs(h);
  if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
  for (cudaEvent_t ev : h->ev_pool) cudaEventDestroy(ev);
  if (h->kick_fork) cudaEventDestroy(h->kick_fork);
  if (h->kick_join) cudaEventDestroy(h->kick_join);
  if (h->kick_stream) cudaStreamDestroy(h->kick_stream);
  free_device(h);
  delete h;
  return GT_OK;
}

int gt_set_stream(gt_handle* h, void* stream) {
  if (!h) return fail(nullptr, GT_ERR_ARG, "gt_set_stream: null handle");
  h->stream = (cudaStream_t)stream;
  return GT_OK;
}

int gt_get_info(const gt_handle* h, gt_info* info) {
  if (!h || !info) return GT_ERR_ARG;
  std::memset(info, 0, sizeof(*info));
  info->n = h->N;
  info->ny = h->NY;
  info->nh = h->NH;
  info->nbin = h->NBIN;
  info->rko = h->rko;
  info->split = h->split;
  info->truncate = h->truncate;
  info->nf = h->nf;
  info->field_doubles = (int64_t)(h->N + 2) * h->NY;
  info->dkx = h->dkx;
  info->dky = h->dky;
  info->inpz = h->inpz;
  info->inpe = h->inpe;
  info->fkxsmax = h->fkxsmax;
  info->fkysmax = h->fkysmax;
  info->rtrunc2 = h->rtrunc2;
  return GT_OK;
}

int gt_get_forcing_modes(const gt_handle* h, int32_t* ikxf, int32_t* ikyf, int32_t* nf) {
  if (!h || !nf) return GT_ERR_ARG;
  *nf = h->nf;
  for (int k = 0; k < h->nf; ++k) {
    if (ikxf) ikxf[k] = h->ikxf[k];
    if (ikyf) ikyf[k] = h->ikyf[k];
  }
  return GT_OK;
}

const char* gt_last_error(const gt_handle* h) {
  return h ? h->err.c_str() : g_create_error.c_str();
}

int gt_sync(gt_handle* h) {
  if (!h) return fail(nullptr, GT_ERR_ARG, "gt_sync: null handle");
  GT_CUDA(h, cudaStreamSynchronize(h->stream));
  GT_CUDA(h, cudaGetLastError());
  return GT_OK;
}

int gt_fft_dir(gt_handle* h, double* z) {
  if (!h || !z) return fail(h, GT_ERR_ARG, "gt_fft_dir: null argument");
  GtOp op = base_op(h);
  op.a = reinterpret_cast<double2*>(z);
  op.kind = gt::OP_ROW_R2C;
  int rc = run(h, op);
  if (rc) return rc;
  op.kind = gt::OP_COL_FWD;
  op.scale = 1.0 / ((double)h->N * (double)h->NY);
  return run(h, op);
}

int gt_fft_inv(gt_handle* h, double* z) {
  if (!h || !z) return fail(h, GT_ERR_ARG, "gt_fft_inv: null argument");
  GtOp op = base_op(h);
  op.a = reinterpret_cast<double2*>(z);
  op.kind = gt::OP_COL_INV;
  int rc = run(h, op);
  if (rc) return rc;
  op.kind = gt::OP_ROW_C2R;
  return run(h, op);
}

int gt_dump_real4(gt_handle* h, double* work, float* out) {
  if (!h || !work || !out) return fail(h, GT_ERR_ARG, "gt_dump_real4: null argument");
  GtOp op = base_op(h);
  op.a = reinterpret_cast<double2*>(work);
  op.kind = gt::OP_COL_INV;
  int rc = run(h, op);
  if (rc) return rc;
  op.f32 = out;
  op.kind = gt::OP_ROW_C2R_F32;
  return run(h, op);
}

int gt_load_real4(gt_handle* h, const float* in, double* z) {
  if (!h || !in || !z) return fail(h, GT_ERR_ARG, "gt_load_real4: null argument");
  GtOp op = base_op(h);
  op.a = reinterpret_cast<double2*>(z);
  op.f32 = const_cast<float*>(in);
  op.kind = gt::OP_ROW_R2C_F32;
  int rc = run(h, op);
  if (rc) return rc;
  op.kind = gt::OP_COL_FWD;
  op.scale = 1.0 / ((double)h->N * (double)h->NY);
  rc = run(h, op);
  if (rc || !h->truncate) return rc;
  return gt_trunc(h, z);
}

int gt_trunc(gt_handle* h, double* z) {
  if (!h || !z) return fail(h, GT_ERR_ARG, "gt_trunc: null argument");
  gt::k_trunc<<<4 * 152, 256, 0, h->stream>>>(reinterpret_cast<double2*>(z), h->NY, h->NH, h->d_kcut);
  GT_CUDA(h, cudaGetLastError());
  return GT_OK;
}

int gt_produ(gt_handle* h, const double* z, double* u, double* v) {
  if (!h || !z || !u || !v) return fail(h, GT_ERR_ARG, "gt_produ: null argument");
  gt::k_produ<<<4 * 152, 256, 0, h->stream>>>(z, u, v, h->N, h->NY);
  GT_CUDA(h, cudaGetLastError());
  return GT_OK;
}

int gt_nlt(gt_handle* h, double* z, double* u, double* v) {
  if (!h || !z || !u || !v) return fail(h, GT_ERR_ARG, "gt_nlt: null argument");
  if (z == u || z == v || u == v) return fail(h, GT_ERR_ARG, "gt_nlt: z, u, v must be distinct");
  return nlt_passes(h, z, z, u, v, make_epi(h, gt::EPI_NLT, z, nullptr, nullptr));
}

// The stages of one Runge-Kutta step: stage k evaluates N at zin[k] (the first from z, the
// others from znl, where the previous stage's epilogue left its value) and applies epi[k].
// Pass C of stage k and pass A of stage k+1 run as one column kernel, or, with the field-split
// column passes, as two (q then goes to the handle's scratch field, since znl is both the next
// stage's input and, in the fused kernel, its q output). The stages alternate between the
// handle's two untruncated-input flags.
int stage_chain(gt_handle* h, int nst, const double* const* zin, double* znl, double* u, double* v,
                const gt::EpiArgs* epi, cudaEvent_t join = nullptr) {
  // the final pass C waits for `join` (the fused kick's increments) when given
  auto await_join = [&](int k) -> int {
    if (!join || k + 1 != nst) return GT_OK;
    const cudaError_t e = cudaStreamWaitEvent(h->stream, join, 0);
    return e == cudaSuccess ? GT_OK : cuda_fail(h, e, "cudaStreamWaitEvent");
  };
  GtOp op = base_op(h);
  const bool split = split_active(h);
  double* qbuf = split ? reinterpret_cast<double*>(h->d_qscr) : znl;
  auto stage = [&](int k) {
    gt::NltArgs a = gt::handle_nlt_args(h, zin[k], qbuf, u, v, h->d_flag + (k & 1));
    a.epi = epi[k];
    return a;
  };
  if (split) {
    // pass A of stage 1, then per stage: pass B, pass C, pass A of the next stage
    op.nlt = stage(0);
    op.kind = gt::OP_NLT_COLINV_FS;
    int rc = run(h, op);
    for (int k = 0; k < nst && !rc; ++k) {
      op.nlt = stage(k);
      op.kind = gt::OP_NLT_ROW;
      rc = run(h, op);
      if (!rc) rc = await_join(k);
      if (!rc) {
        op.kind = gt::OP_NLT_COLFWD_FS;
        rc = run(h, op);
      }
      if (!rc && k + 1 < nst) {
        op.nlt = stage(k + 1);
        op.kind = gt::OP_NLT_COLINV_FS;
        rc = run(h, op);
      }
    }
    return rc;
  }
  op.nlt = stage(0);
  op.kind = gt::OP_NLT_COLINV;
  int rc = run(h, op);
  for (int k = 0; k < nst && !rc; ++k) {
    op.nlt = stage(k);
    op.kind = gt::OP_NLT_ROW;
    rc = run(h, op);
    if (rc) break;
    if (k + 1 < nst) {
      op.nlt2 = stage(k + 1);
      op.kind = gt::OP_NLT_COLFWD_INV;
    } else {
      op.kind = gt::OP_NLT_COLFWD;
      rc = await_join(k);
      if (rc) break;
    }
    rc = run(h, op);
  }
  return rc;
}

static int step_rk2_direct(gt_handle* h, double* z, double* znl, double* u, double* v) {
  const gt::EpiArgs epi[2] = {make_epi(h, gt::EPI_RK2A, znl, nullptr, z),
                              make_epi(h, gt::EPI_RK2B, z, nullptr, z)};
  const double* zin[2] = {z, znl};
  return stage_chain(h, 2, zin, znl, u, v, epi);
}

static int step_rk4_direct(gt_handle* h, double* z, double* znl, double* znew, double* u, double* v) {
  const gt::EpiArgs epi[4] = {make_epi(h, gt::EPI_RK4A, znl, znew, z), make_epi(h, gt::EPI_RK4B, znl, znew, z),
                              make_epi(h, gt::EPI_RK4C, znl, znew, z), make_epi(h, gt::EPI_RK4D, z, znew, nullptr)};
  const double* zin[4] = {z, znl, znl, znl};
  return stage_chain(h, 4, zin, znl, u, v, epi);
}

// The final stage's fused kick from LCG state x0 (forcing.f90:16-33): the nf increments are
// computed on a side stream that forks from the handle's stream before the step, and the final
// pass C waits for them (the returned event). The sincos of the phases thus stays off the
// final pass's critical path.
// the side stream and events of the fused kick, made once per handle (before any capture)
static int ensure_kick_stream(gt_handle* h) {
  if (h->kick_stream) return GT_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&h->kick_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->kick_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->kick_join, cudaEventDisableTiming);
  return e == cudaSuccess ? GT_OK : cuda_fail(h, e, "fused kick: stream set-up");
}

static int start_fused_kick(gt_handle* h, gt::EpiArgs& E, uint32_t x0, cudaEvent_t* join) {
  int rc = ensure_kick_stream(h);
  if (rc) return rc;
  cudaError_t e = cudaEventRecord(h->kick_fork, h->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(h->kick_stream, h->kick_fork, 0);
  if (e != cudaSuccess) return cuda_fail(h, e, "fused kick: fork");
  gt::k_kick_values<<<(h->nf + 127) / 128, 128, 0, h->kick_stream>>>(h->d_kick, h->nf, h->d_lcga, h->d_lcgb,
                                                                       h->d_ff, x0, h->sdt * h->p.famp);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventRecord(h->kick_join, h->kick_stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "fused kick: increments");
  E.fmap = h->d_fmap;
  E.fwi = h->fwi;
  E.fwj = h->fwj;
  E.fh = h->fh;
  E.kick = h->d_kick;
  *join = h->kick_join;
  return GT_OK;
}

// RK2 step with the kick fused into its final stage, from LCG state x0 (nf > 0, fuse_ok)
static int step_rk2_forced_direct(gt_handle* h, double* z, double* znl, double* u, double* v, uint32_t x0) {
  gt::EpiArgs epi[2] = {make_epi(h, gt::EPI_RK2A, znl, nullptr, z),
                        make_epi(h, gt::EPI_RK2B, z, nullptr, z)};
  cudaEvent_t join = nullptr;
  int rc = start_fused_kick(h, epi[1], x0, &join);
  if (rc) return rc;
  const double* zin[2] = {z, znl};
  return stage_chain(h, 2, zin, znl, u, v, epi, join);
}

static int step_rk4_forced_direct(gt_handle* h, double* z, double* znl, double* znew, double* u, double* v,
                                  uint32_t x0) {
  gt::EpiArgs epi[4] = {make_epi(h, gt::EPI_RK4A, znl, znew, z), make_epi(h, gt::EPI_RK4B, znl, znew, z),
                        make_epi(h, gt::EPI_RK4C, znl, znew, z), make_epi(h, gt::EPI_RK4D, z, znew, nullptr)};
  cudaEvent_t join = nullptr;
  int rc = start_fused_kick(h, epi[3], x0, &join);
  if (rc) return rc;
  const double* zin[4] = {z, znl, znl, znl};
  return stage_chain(h, 4, zin, znl, u, v, epi, join);
}

// ---- steps as CUDA graphs ---------------------------------------------------------------
// A step is a dozen short launches. Each step kind is captured once per (fields, launch
// settings) into a CUDA graph on a capture stream of the handle and replayed on the handle's
// stream as one launch, which takes the per-launch host work off the step (at 256^2 RK4 the GPU
// time of the kernels, about 0.1 ms, still sets the step time). The graph holds the same
// launches with the same arguments, so its results are the direct launches' bit for bit. The
// forced steps' kick increments depend on the LCG state of the call: the k_kick_values node's
// parameters are rewritten before each replay.
enum StepKind { SK_RK2 = 1, SK_RK4 = 2, SK_RK2F = 3, SK_RK4F = 4 };
constexpr size_t kStepGraphs = 8;

static int step_direct(gt_handle* h, int kind, double* const* f, uint32_t x0) {
  switch (kind) {
    case SK_RK2: return step_rk2_direct(h, f[0], f[1], f[3], f[4]);
    case SK_RK4: return step_rk4_direct(h, f[0], f[1], f[2], f[3], f[4]);
    case SK_RK2F: return step_rk2_forced_direct(h, f[0], f[1], f[3], f[4], x0);
    default: return step_rk4_forced_direct(h, f[0], f[1], f[2], f[3], f[4], x0);
  }
}

static void free_step_graph(gt_handle::StepGraph& g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.graph) cudaGraphDestroy(g.graph);
  g.exec = nullptr;
  g.graph = nullptr;
}

static void drop_step_graphs(gt_handle* h) {
  for (auto& g : h->sg) free_step_graph(g);
  h->sg.clear();
}

// the kick kernel's parameters for LCG state x0 (the k_kick_values launch of start_fused_kick)
static cudaError_t set_kick_node(gt_handle* h, cudaGraphExec_t exec, cudaGraphNode_t node, uint32_t x0) {
  double2* kick = h->d_kick;
  int nf = h->nf;
  const uint32_t* lcga = h->d_lcga;
  const uint32_t* lcgb = h->d_lcgb;
  const double2* ff = h->d_ff;
  uint32_t seed0 = x0;
  double sf = h->sdt * h->p.famp;
  void* args[] = {&kick, &nf, &lcga, &lcgb, &ff, &seed0, &sf};
  cudaKernelNodeParams kp = {};
  kp.func = (void*)gt::k_kick_values;
  kp.gridDim = dim3((unsigned)((h->nf + 127) / 128));
  kp.blockDim = dim3(128);
  kp.sharedMemBytes = 0;
  kp.kernelParams = args;
  kp.extra = nullptr;
  return cudaGraphExecKernelNodeSetParams(exec, node, &kp);
}

// Captures one step of `kind` on the fields f; on success *out holds the instantiated graph.
static int capture_step(gt_handle* h, int kind, double* const* f, uint32_t x0, gt_handle::StepGraph* out) {
  cudaError_t e = cudaSuccess;
  if (!h->cap_stream) {
    e = cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(h, e, "step graph: capture stream");
  }
  if ((kind == SK_RK2F || kind == SK_RK4F) && ensure_kick_stream(h)) return GT_ERR_CUDA;
  cudaStream_t saved = h->stream;
  h->stream = h->cap_stream;
  e = cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    h->stream = saved;
    return cuda_fail(h, e, "step graph: cudaStreamBeginCapture");
  }
  const int rc = step_direct(h, kind, f, x0);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(h->cap_stream, &graph);
  h->stream = saved;
  if (rc || e != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return rc ? rc : cuda_fail(h, e == cudaSuccess ? cudaErrorStreamCaptureInvalidated : e, "step graph: capture");
  }
  // the kick node of a forced step
  cudaGraphNode_t kick = nullptr;
  if (kind == SK_RK2F || kind == SK_RK4F) {
    size_t nn = 0;
    e = cudaGraphGetNodes(graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (e == cudaSuccess && nn) e = cudaGraphGetNodes(graph, nodes.data(), &nn);
    for (size_t k = 0; k < nn && e == cudaSuccess && !kick; ++k) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nodes[k], &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
      cudaKernelNodeParams kp = {};
      if (cudaGraphKernelNodeGetParams(nodes[k], &kp) == cudaSuccess && kp.func == (void*)gt::k_kick_values)
        kick = nodes[k];
    }
    if (e != cudaSuccess || !kick) {
      cudaGraphDestroy(graph);
      cudaGetLastError();
      return cuda_fail(h, e == cudaSuccess ? cudaErrorInvalidValue : e, "step graph: kick node");
    }
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    cudaGetLastError();
    return cuda_fail(h, e, "step graph: cudaGraphInstantiate");
  }
  out->graph = graph;
  out->exec = exec;
  out->kick = kick;
  return GT_OK;
}

// One step of `kind`: replayed from its graph where graphs are on, else launched directly.
static int run_step(gt_handle* h, int kind, double* z, double* znl, double* znew, double* u, double* v, uint32_t x0) {
  double* const f[5] = {z, znl, znew, u, v};
  bool use = h->graphs && !h->prof && !h->graph_failed;
  if (use) {  // a step enqueued into a stream that is itself being captured stays a set of launches
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(h->stream, &cs) != cudaSuccess) {
      cudaGetLastError();
      use = false;
    } else if (cs != cudaStreamCaptureStatusNone) {
      use = false;
    }
  }
  if (!use) return step_direct(h, kind, f, x0);
  gt_handle::StepGraph* g = nullptr;
  for (auto& c : h->sg) {
    if (c.kind == kind && c.variant == h->variant && c.row_variant == h->row_variant &&
        c.col_split == h->col_split && c.pdl == h->pdl && c.f[0] == z && c.f[1] == znl && c.f[2] == znew &&
        c.f[3] == u && c.f[4] == v) {
      g = &c;
      break;
    }
  }
  if (!g) {
    gt_handle::StepGraph ng;
    ng.kind = kind;
    for (int k = 0; k < 5; ++k) ng.f[k] = f[k];
    ng.variant = h->variant;
    ng.row_variant = h->row_variant;
    ng.col_split = h->col_split;
    ng.pdl = h->pdl;
    const int rc = capture_step(h, kind, f, x0, &ng);
    if (rc) {  // graphs unavailable here: direct launches from now on
      h->graph_failed = true;
      h->err.clear();
      return step_direct(h, kind, f, x0);
    }
    // a handle that cycles through more field sets than it keeps graphs for would capture on
    // almost every step: after 16 captures with fewer than two replays each, launch directly
    if (++h->sg_captures >= 16 && h->sg_replays < 2 * h->sg_captures) {
      free_step_graph(ng);
      drop_step_graphs(h);
      h->graph_failed = true;
      return step_direct(h, kind, f, x0);
    }
    if (h->sg.size() >= kStepGraphs) {  // evict the least recently used
      size_t lru = 0;
      for (size_t k = 1; k < h->sg.size(); ++k)
        if (h->sg[k].used < h->sg[lru].used) lru = k;
      free_step_graph(h->sg[lru]);
      h->sg.erase(h->sg.begin() + (long)lru);
    }
    h->sg.push_back(ng);
    g = &h->sg.back();
  }
  g->used = ++h->sg_clock;
  ++h->sg_replays;
  cudaError_t e = cudaSuccess;
  if (g->kick) e = set_kick_node(h, g->exec, g->kick, x0);
  if (e == cudaSuccess) e = cudaGraphLaunch(g->exec, h->stream);
  if (e != cudaSuccess) {  // nothing was enqueued: direct launches from now on
    cudaGetLastError();
    drop_step_graphs(h);
    h->graph_failed = true;
    return step_direct(h, kind, f, x0);
  }
  return GT_OK;
}

int gt_step_rk2(gt_handle* h, double* z, double* znl, double* u, double* v) {
  if (!h || !z || !znl || !u || !v) return fail(h, GT_ERR_ARG, "gt_step_rk2: null argument");
  return run_step(h, SK_RK2, z, znl, nullptr, u, v, 0);
}

int gt_step_rk4(gt_handle* h, double* z, double* znl, double* znew, double* u, double* v) {
  if (!h || !z || !znl || !znew || !u || !v) return fail(h, GT_ERR_ARG, "gt_step_rk4: null argument");
  if (h->split) return fail(h, GT_ERR_ARG, "gt_step_rk4: the split integrator exists only for RK2");
  return run_step(h, SK_RK4, z, znl, znew, u, v, 0);
}

int gt_step_rk2_forced(gt_handle* h, double* z, double* znl, double* u, double* v, int32_t* seed) {
  if (!h || !z || !znl || !u || !v || !seed) return fail(h, GT_ERR_ARG, "gt_step_rk2_forced: null argument");
  if (!(h->nf > 0 && h->fuse_ok)) {
    const int rc = gt_step_rk2(h, z, znl, u, v);
    return rc ? rc : gt_forcing(h, z, seed);
  }
  const uint32_t x0 = (uint32_t)(*seed);
  const int rc = run_step(h, SK_RK2F, z, znl, nullptr, u, v, x0);
  if (rc) return rc;
  *seed = (int32_t)((h->lcga_nf * x0 + h->lcgb_nf) & 0x7FFFFFFFu);
  return GT_OK;
}

int gt_step_rk4_forced(gt_handle* h, double* z, double* znl, double* znew, double* u, double* v,
                       int32_t* seed) {
  if (!h || !z || !znl || !znew || !u || !v || !seed)
    return fail(h, GT_ERR_ARG, "gt_step_rk4_forced: null argument");
  if (h->split) return fail(h, GT_ERR_ARG, "gt_step_rk4_forced: the split integrator exists only for RK2");
  if (!(h->nf > 0 && h->fuse_ok)) {
    const int rc = gt_step_rk4(h, z, znl, znew, u, v);
    return rc ? rc : gt_forcing(h, z, seed);
  }
  const uint32_t x0 = (uint32_t)(*seed);
  const int rc = run_step(h, SK_RK4F, z, znl, znew, u, v, x0);
  if (rc) return rc;
  *seed = (int32_t)((h->lcga_nf * x0 + h->lcgb_nf) & 0x7FFFFFFFu);
  return GT_OK;
}

int gt_set_graphs(gt_handle* h, int32_t on) {
  if (!h) return fail(nullptr, GT_ERR_ARG, "gt_set_graphs: null handle");
  h->graphs = on ? 1 : 0;
  if (!on) drop_step_graphs(h);
  h->graph_failed = false;
  h->sg_captures = h->sg_replays = 0;
  return GT_OK;
}

int gt_get_graphs(const gt_handle* h, int32_t* on) {
  if (!h || !on) return fail(nullptr, GT_ERR_ARG, "gt_get_graphs: null argument");
  *on = h->graphs && !h->graph_failed;
  return GT_OK;
}

float gt_rann(int32_t* seed) {
  uint32_t x = (uint32_t)(*seed);
  x = (69069u * x + 1u) & 0x7FFFFFFFu;
  *seed = (int32_t)x;
  return (float)((double)x / (double)0x7FFFFFFF);
}

int gt_forcing(gt_handle* h, double* z, int32_t* seed) {
  if (!h || !z || !seed) return fail(h, GT_ERR_ARG, "gt_forcing: null argument");
  if (h->nf == 0) return GT_OK;
  const uint32_t x0 = (uint32_t)(*seed);
  const double sf = h->sdt * h->p.famp;
  const int pair = prof_begin(h, GT_PROF_FORCING);
  gt::k_forcing<<<(h->nf + 127) / 128, 128, 0, h->stream>>>(
      reinterpret_cast<double2*>(z), h->NH, h->nf, h->d_ikxf, h->d_ikyf, h->d_jc, h->d_lcga,
      h->d_lcgb, h->d_ff, x0, sf);
  prof_end(h, pair);
  GT_CUDA(h, cudaGetLastError());
  *seed = (int32_t)((h->lcga_nf * x0 + h->lcgb_nf) & 0x7FFFFFFFu);
  return GT_OK;
}

int gt_diag(gt_handle* h, const double* z, const double* znl, double* sp, double* sz, double* fle,
            double* flz, double* glob) {
  if (!h || !z) return fail(h, GT_ERR_ARG, "gt_diag: null argument");
  if ((fle || flz) && !znl) return fail(h, GT_ERR_ARG, "gt_diag: fluxes need znl");
  gt::DiagArgs D;
  D.z = reinterpret_cast<const double2*>(z);
  D.znl = reinterpret_cast<const double2*>(znl);
  D.fkxs = h->d_fkxs;
  D.fkys = h->d_fkys;
  D.kainv = h->d_kainv;
  D.n = h->NY;  // rows
  D.nh = h->NH;
  D.nbin = h->NBIN;
  D.dk = h->dkx;
  D.unit_k = (h->dkx == 1.0 && h->dky == 1.0) ? 1 : 0;
  D.alpv = h->p.alpv;
  D.nu = h->p.nu;
  D.mu = h->p.mu;
  D.alpnu = h->p.alpnu;
  D.alpmu = h->p.alpmu;
  D.inu = gt::diag_int_exponent(h->p.alpnu);
  D.imu = gt::diag_int_exponent(h->p.alpmu);
  D.part = h->d_part;
  D.rowsum = h->d_rowsum;
  const int nb = h->NBIN;
  double* hb = h->h_diag;
  double* hf = hb + (size_t)nb * 4;
  double* hg = hf + (size_t)nb * 2;
  const bool want_bins = sp || sz || fle || flz;
  const int pair = prof_begin(h, GT_PROF_DIAG);
  if (want_bins) {
    gt::diag_launch_bins(D, h->stream);
    gt::k_diag_bins_final<<<(nb + 127) / 128, 128, 0, h->stream>>>(D, h->d_bins);
    GT_CUDA(h, cudaGetLastError());
    GT_CUDA(h, cudaMemcpyAsync(hb, h->d_bins, sizeof(double) * nb * 4, cudaMemcpyDeviceToHost, h->stream));
    if (znl) {
      gt::k_diag_suffix<<<1, gt::kDiagThreads, gt::diag_suffix_smem(nb), h->stream>>>(h->d_bins, h->d_fl, nb);
      GT_CUDA(h, cudaGetLastError());
      GT_CUDA(h, cudaMemcpyAsync(hf, h->d_fl, sizeof(double) * nb * 2, cudaMemcpyDeviceToHost, h->stream));
    }
  }
  if (glob) {
    gt::k_diag_glob_rows<<<h->NY, 256, 0, h->stream>>>(D);
    gt::k_diag_glob_final<<<1, 192, 0, h->stream>>>(D, h->d_glob);
    GT_CUDA(h, cudaGetLastError());
    GT_CUDA(h, cudaMemcpyAsync(hg, h->d_glob, sizeof(double) * 6, cudaMemcpyDeviceToHost, h->stream));
  }
  prof_end(h, pair);
  GT_CUDA(h, cudaStreamSynchronize(h->stream));
  for (int b = 0; b < nb; ++b) {
    if (sp) sp[b] = hb[b * 4 + 0];
    if (sz) sz[b] = hb[b * 4 + 1];
    if (fle) fle[b] = hf[b * 2 + 0];
    if (flz) flz[b] = hf[b * 2 + 1];
  }
  if (glob) {
    bool finite = true;
    for (int q = 0; q < 6; ++q) {
      glob[q] = hg[q];
      finite = finite && std::isfinite(hg[q]);
    }
    if (!finite) return fail(h, GT_ERR_NONFINITE, "gt_diag: non-finite global budget");
  }
  return GT_OK;
}

int gt_profile(gt_handle* h, int enable) {
  if (!h) return fail(nullptr, GT_ERR_ARG, "gt_profile: null handle");
  h->prof = enable != 0;
  return GT_OK;
}

int gt_profile_read(gt_handle* h, double* ms, int64_t* launches) {
  if (!h || !ms || !launches) return fail(h, GT_ERR_ARG, "gt_profile_read: null argument");
  GT_CUDA(h, cudaStreamSynchronize(h->stream));
  for (int k = 0; k < GT_PROF_KINDS; ++k) {
    ms[k] = 0.0;
    launches[k] = 0;
  }
  for (size_t p = 0; p < h->ev_kind.size(); ++p) {
    float t = 0.0f;
    GT_CUDA(h, cudaEventElapsedTime(&t, h->ev_pool[2 * p], h->ev_pool[2 * p + 1]));
    ms[h->ev_kind[p]] += t;
    launches[h->ev_kind[p]] += 1;
  }
  h->ev_kind.clear();
  return GT_OK;
}

int gt_set_col_split(gt_handle* h, int32_t on) {
  if (!h) return fail(nullptr, GT_ERR_ARG, "gt_set_col_split: null handle");
  h->col_split = on <= 0 ? 0 : on >= 2 ? 2 : 1;
  return GT_OK;
}

int gt_set_pdl(gt_handle* h, int32_t on) {
  if (!h) return fail(nullptr, GT_ERR_ARG, "gt_set_pdl: null handle");
  h->pdl = on ? 1 : 0;
  return GT_OK;
}

int gt_get_pdl(const gt_handle* h, int32_t* on) {
  if (!h || !on) return fail(nullptr, GT_ERR_ARG, "gt_get_pdl: null argument");
  *on = h->pdl;
  return GT_OK;
}

int gt_adj_set_memory(gt_handle* h, int64_t bytes) {
  if (!h) return fail(nullptr, GT_ERR_ARG, "gt_adj_set_memory: null handle");
  if (bytes < 0) return fail(h, GT_ERR_ARG, "gt_adj_set_memory: negative budget");
  h->adj_mem = bytes;
  return GT_OK;
}

int gt_adj_get_memory(const gt_handle* h, int64_t* bytes) {
  if (!h || !bytes) return fail(nullptr, GT_ERR_ARG, "gt_adj_get_memory: null argument");
  *bytes = h->adj_mem;
  return GT_OK;
}

int gt_get_col_split(const gt_handle* h, int32_t* active) {
  if (!h || !active) return fail(nullptr, GT_ERR_ARG, "gt_get_col_split: null argument");
  *active = split_active(h) ? h->col_split : 0;
  return GT_OK;
}

int gt_variant_supported(int32_t n, int32_t variant) {
  if (!pow2_in_range(n)) return 0;
  switch (variant) {
    case 0: return 1;
    case 1: return n <= 8192;
    case 2:
    case 3:
    case 4: return n <= 1024;
    case 5: return n >= 32 && n <= 512;
    default: return 0;
  }
}

int gt_row_variant_supported(int32_t n, int32_t row_variant) {
  return row_variant >= 0 && row_variant < GT_NROW_VARIANTS && gt_variant_supported(n, row_variant);
}
static_assert(GT_NROW_VARIANTS == GT_NVARIANTS, "row and column variants share their numbering");

int gt_set_variants(gt_handle* h, int32_t col_variant, int32_t row_variant) {
  if (!h) return fail(nullptr, GT_ERR_ARG, "gt_set_variants: null handle");
  if (!col_variant_ok(h, col_variant) || !gt_row_variant_supported(h->N, row_variant))
    return fail(h, GT_ERR_ARG, "gt_set_variants: variants (" + std::to_string(col_variant) + ", " +
                                   std::to_string(row_variant) + ") do not exist for the " + std::to_string(h->N) +
                                   " x " + std::to_string(h->NY) + " grid (columns of length NY, rows of NX)");
  h->variant = col_variant;
  h->row_variant = row_variant;
  return GT_OK;
}

int gt_set_variant(gt_handle* h, int32_t variant) {
  if (!h) return fail(nullptr, GT_ERR_ARG, "gt_set_variant: null handle");
  if (!col_variant_ok(h, variant) || !gt_row_variant_supported(h->N, natural_row_variant(variant)))
    return fail(h, GT_ERR_ARG, "gt_set_variant: variant " + std::to_string(variant) + " does not exist for the " +
                                   std::to_string(h->N) + " x " + std::to_string(h->NY) + " grid");
  return gt_set_variants(h, variant, natural_row_variant(variant));
}

int gt_get_variant(const gt_handle* h, int32_t* variant) {
  if (!h || !variant) return fail(nullptr, GT_ERR_ARG, "gt_get_variant: null argument");
  *variant = h->variant;
  return GT_OK;
}

int gt_get_variants(const gt_handle* h, int32_t* col_variant, int32_t* row_variant) {
  if (!h || !col_variant || !row_variant) return fail(nullptr, GT_ERR_ARG, "gt_get_variants: null argument");
  *col_variant = h->variant;
  *row_variant = h->row_variant;
  return GT_OK;
}

int gt_autotune(gt_handle* h, int32_t steps, double* ms_per_step, int32_t* best) {
  if (!h) return fail(nullptr, GT_ERR_ARG, "gt_autotune: null handle");
  if (steps < 1) return fail(h, GT_ERR_ARG, "gt_autotune: steps must be >= 1");
  double ms[GT_NVARIANTS];
  int navail = 0;
  for (int v = 0; v < GT_NVARIANTS; ++v) {
    ms[v] = -1.0;
    navail += col_variant_ok(h, v) + gt_row_variant_supported(h->N, v);
  }
  if (navail > 2) {
    const size_t nd = (size_t)h->NY * (size_t)(h->N + 2);
    double* buf = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    const int saved_col = h->variant, saved_row = h->row_variant;
    const bool prof = h->prof;
    h->prof = false;
    int rc = GT_OK;
    cudaError_t e = cudaMalloc((void**)&buf, 5 * nd * sizeof(double));
    if (e != cudaSuccess) rc = cuda_fail(h, e, "gt_autotune: cudaMalloc");
    if (!rc) e = cudaMemsetAsync(buf, 0, 5 * nd * sizeof(double), h->stream);
    if (!rc && e == cudaSuccess) e = cudaEventCreate(&ev[0]);
    if (!rc && e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    if (!rc && e != cudaSuccess) rc = cuda_fail(h, e, "gt_autotune: set-up");
    double* f[5];
    for (int k = 0; k < 5; ++k) f[k] = buf ? buf + k * nd : nullptr;
    auto one_step = [&]() {
      return h->rko == 4 ? gt_step_rk4(h, f[0], f[1], f[2], f[3], f[4]) : gt_step_rk2(h, f[0], f[1], f[3], f[4]);
    };
    // ms per step of (column variant c, row variant r), or -1 on failure
    auto time_pair = [&](int c, int r) -> double {
      h->variant = c;
      h->row_variant = r;
      for (int w = 0; w < 3 && !rc; ++w) rc = one_step();
      if (!rc) e = cudaEventRecord(ev[0], h->stream);
      for (int s = 0; s < steps && !rc; ++s) rc = one_step();
      if (!rc && e == cudaSuccess) e = cudaEventRecord(ev[1], h->stream);
      if (!rc && e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
      float t = 0.0f;
      if (!rc && e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
      if (!rc && e != cudaSuccess) rc = cuda_fail(h, e, "gt_autotune: timing");
      return rc ? -1.0 : (double)t / steps;
    };
    // stage 1: every column variant with the row tiles of its own register radix (the handle's
    // row variant where the row length has no such variant)
    int best_c = 0;
    auto row_for = [&](int v) { return gt_row_variant_supported(h->N, natural_row_variant(v)) ? natural_row_variant(v)
                                                                                             : saved_row; };
    for (int v = 0; v < GT_NVARIANTS && !rc; ++v) {
      if (!col_variant_ok(h, v)) continue;
      ms[v] = time_pair(v, row_for(v));
      if (!rc && (ms[best_c] < 0.0 || ms[v] < ms[best_c])) best_c = v;
    }
    // stage 2: every row variant under each of the two fastest column variants (a column
    // variant's own row tiles need not be its best partner); ms[c] becomes column variant c's
    // best time over the rows tried with it
    int cand[2] = {best_c, -1};
    for (int v = 0; v < GT_NVARIANTS; ++v)
      if (v != best_c && ms[v] >= 0.0 && (cand[1] < 0 || ms[v] < ms[cand[1]])) cand[1] = v;
    int best_r = row_for(best_c);
    double best_ms = ms[best_c];
    for (int ci = 0; ci < 2 && !rc; ++ci) {
      const int c = cand[ci];
      if (c < 0) continue;
      for (int r = 0; r < GT_NROW_VARIANTS && !rc; ++r) {
        if (r == row_for(c) || !gt_row_variant_supported(h->N, r)) continue;
        const double t = time_pair(c, r);
        if (rc || t < 0.0) break;
        if (t < ms[c]) ms[c] = t;
        if (t < best_ms) {
          best_ms = t;
          best_c = c;
          best_r = r;
        }
      }
    }
    // stage 3: the best pair with one CTA per column, where the field-split passes ran
    h->variant = best_c;
    if (!rc && h->col_split && split_active(h)) {
      const int mode = h->col_split;
      h->col_split = 0;
      const double t = time_pair(best_c, best_r);
      if (rc || !(t < best_ms)) h->col_split = mode;
    }
    if (buf) {
      cudaStreamSynchronize(h->stream);
      cudaFree(buf);
    }
    for (cudaEvent_t x : ev)
      if (x) cudaEventDestroy(x);
    h->prof = prof;
    h->variant = rc ? saved_col : best_c;
    h->row_variant = rc ? saved_row : best_r;
    if (rc) return rc;
  }
  if (ms_per_step)
    for (int v = 0; v < GT_NVARIANTS; ++v) ms_per_step[v] = ms[v];
  if (best) *best = h->variant;
  return GT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// gt_diag_static: the diagnostics without any device allocation.
//
// For callers that cannot allocate device memory: a driver whose device arrays all live in
// OpenACC data regions (the reference's main program) or in another runtime's memory pool,
// sized to fill the GPU, and host code that must not call cudaMalloc/cudaFree between time
// steps, because those calls synchronise the whole device. Such a caller has no gt_handle
// (gt_create allocates the tables) and passes only its fields and output arrays.
//
// The scratch (partial shell sums, per-row budgets, the k^2 tables) is this file-scope device
// array, present on every GPU that loads the library until the process exits. Host code
// reaches it only through the address that cudaGetSymbolAddress returns for the current
// device. Every call made outside a stream capture looks that address up again (a device reset
// between calls is therefore harmless); a call made while its stream captures reuses the
// address of the device's last earlier call, so the first call on each device should be made
// before any stream capture. Every call rewrites all the scratch it reads, so nothing
// has to start at zero; calls that overlap on the GPU (other streams, other threads) share
// the array and race.
// ---------------------------------------------------------------------------------------
namespace {

constexpr int kStaticMaxN = GT_DIAG_STATIC_MAX_N;
constexpr int kStaticMaxNH = kStaticMaxN / 2 + 1;
constexpr int kStaticMaxBin = kStaticMaxN / 2;
constexpr int kStaticGroups = gt::diag_groups(kStaticMaxN);
constexpr size_t kOffFkxs = 0;
constexpr size_t kOffFkys = kOffFkxs + ((kStaticMaxNH + 31) / 32) * 32;
constexpr size_t kOffPart = kOffFkys + kStaticMaxN;
constexpr size_t kOffRows = kOffPart + (size_t)kStaticGroups * kStaticMaxBin * 4;
constexpr size_t kOffBins = kOffRows + (size_t)kStaticMaxN * 6;
constexpr size_t kOffFl = kOffBins + (size_t)kStaticMaxBin * 4;
constexpr size_t kStaticDoubles = kOffFl + (size_t)kStaticMaxBin * 2;

static __device__ __align__(256) double g_diag_scratch[kStaticDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
double* g_static_ptr[kMaxDevices] = {nullptr};

// (i dkx)^2 and (fky(j))^2 exactly as defk.f90:27-43 forms them.
__global__ void k_static_k2(double* fkxs, double* fkys, int n, double dkx, double dky) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n / 2 + 1) {
    const double kx = (double)t * dkx;
    fkxs[t] = kx * kx;
  }
  if (t < n) {
    const double ky = (double)(t <= n / 2 ? t : t - n) * dky;
    fkys[t] = ky * ky;
  }
}

__global__ void k_static_scatter(const double* bins, const double* fl, double* sp, double* sz,
                                 double* fle, double* flz, int nbin) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbin) return;
  if (sp) sp[b] = bins[b * 4 + 0];
  if (sz) sz[b] = bins[b * 4 + 1];
  if (fle) fle[b] = fl[b * 2 + 0];
  if (flz) flz[b] = fl[b * 2 + 1];
}

}  // namespace

extern "C" int gt_diag_static(const gt_params* p, const double* z, const double* znl, double* sp,
                              double* sz, double* fle, double* flz, double* glob,
                              void* cuda_stream) {
  if (!p || !z) return fail(nullptr, GT_ERR_ARG, "gt_diag_static: null argument");
  const int n = p->n;
  if (n < 16 || (n & (n - 1)) || n > kStaticMaxN)
    return fail(nullptr, GT_ERR_ARG,
                "gt_diag_static: n must be a power of two in [16, GT_DIAG_STATIC_MAX_N=2048]");
  if ((fle || flz) && !znl) return fail(nullptr, GT_ERR_ARG, "gt_diag_static: fluxes need znl");
  if (p->ny != 0 && p->ny != n) return fail(nullptr, GT_ERR_ARG, "gt_diag_static: square grids only (ny = 0 or n)");
  if (!(p->xlx > 0.0) || !(p->xly > 0.0))
    return fail(nullptr, GT_ERR_ARG, "gt_diag_static: xlx and xly must be positive");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "gt_diag_static: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(nullptr, GT_ERR_ARG, "gt_diag_static: device index");
  cudaStream_t s = (cudaStream_t)cuda_stream;
  cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(s, &capturing);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "gt_diag_static: cudaStreamIsCapturing");
  double* base;
  {
    // Outside a capture the address is looked up on every call, so a device reset or a
    // re-created primary context between calls leaves no stale address behind. A call on a
    // capturing stream reuses the address of the device's last earlier call.
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (capturing == cudaStreamCaptureStatusNone) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_diag_scratch);
      if (e != cudaSuccess) return cuda_fail(nullptr, e, "gt_diag_static: cudaGetSymbolAddress");
      g_static_ptr[dev] = static_cast<double*>(ptr);
    } else if (!g_static_ptr[dev]) {
      return fail(nullptr, GT_ERR_STATE,
                  "gt_diag_static: first call on this device made during a stream capture");
    }
    base = g_static_ptr[dev];
  }
  const int nh = n / 2 + 1, nb = n / 2;
  gt::DiagArgs D;
  D.z = reinterpret_cast<const double2*>(z);
  D.znl = reinterpret_cast<const double2*>(znl);
  D.fkxs = base + kOffFkxs;
  D.fkys = base + kOffFkys;
  D.kainv = nullptr;
  D.n = n;
  D.nh = nh;
  D.nbin = nb;
  D.dk = 2.0 * 3.14159265358979323846 / p->xlx;
  D.alpv = p->alpv;
  D.nu = p->nu;
  D.mu = p->mu;
  D.alpnu = p->alpnu;
  D.alpmu = p->alpmu;
  D.inu = gt::diag_int_exponent(p->alpnu);
  D.imu = gt::diag_int_exponent(p->alpmu);
  D.part = base + kOffPart;
  D.rowsum = base + kOffRows;
  const double dky = 2.0 * 3.14159265358979323846 / p->xly;
  D.unit_k = (D.dk == 1.0 && dky == 1.0) ? 1 : 0;
  k_static_k2<<<(n + 127) / 128, 128, 0, s>>>(base + kOffFkxs, base + kOffFkys, n, D.dk, dky);
  if (sp || sz || fle || flz) {
    gt::diag_launch_bins(D, s);
    gt::k_diag_bins_final<<<(nb + 127) / 128, 128, 0, s>>>(D, base + kOffBins);
    if (znl) gt::k_diag_suffix<<<1, gt::kDiagThreads, gt::diag_suffix_smem(nb), s>>>(base + kOffBins, base + kOffFl, nb);
    k_static_scatter<<<(nb + 127) / 128, 128, 0, s>>>(base + kOffBins, base + kOffFl, sp, sz,
                                                       znl ? fle : nullptr, znl ? flz : nullptr, nb);
  }
  if (glob) {
    gt::k_diag_glob_rows<<<n, 256, 0, s>>>(D);
    gt::k_diag_glob_final<<<1, 192, 0, s>>>(D, glob);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "gt_diag_static: launch");
  return GT_OK;
}
