// gt_adj.cu -- tangent-linear model and discrete adjoint of the Lawson RK2 and RK4 steps with
// the LCG forcing kick, and the checkpointed gradient driver (no counterpart in the reference).
//
// Objective: J(z) = sum over kmin <= |k| <= kmax of fac |z|^2 / |k|^alpha, the reference's
// energy weights (fac = 1/2 on the kx=0 and Nyquist columns, src/diagnostics.f90:150-156).
// Parameters: the state entries (real and imaginary parts of the stored half-spectrum) and the
// forcing amplitude famp; the forcing phases are the reference's LCG sequence from a seed.
#include <cuda_runtime.h>

#include <algorithm>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gturbo.h"
#include "gt_internal.h"
#include "gt_ops.h"

namespace gt {

// per-row partial sums of J (and its gradient), fixed-order tree reduction
__global__ void k_objective_rows(const double2* __restrict__ z, const double* __restrict__ fkxs,
                                 const double* __restrict__ fkys, const double* __restrict__ kainv,
                                 int nh, double k2lo, double k2hi, double* rowsum, double2* grad) {
  const int j = blockIdx.x;
  double acc = 0.0;
  const double ky2 = fkys[j];
  for (int i = threadIdx.x; i < nh; i += blockDim.x) {
    const size_t o = (size_t)j * nh + i;
    const double k2 = fkxs[i] + ky2;
    const bool in = k2 >= k2lo && k2 <= k2hi && !(i == 0 && j == 0);
    const double fac = (i == 0 || i == nh - 1) ? 0.5 : 1.0;
    const double2 q = z[o];
    const double w = in ? fac * kainv[o] : 0.0;
    acc += w * (q.x * q.x + q.y * q.y);
    if (grad) grad[o] = make_double2(2.0 * w * q.x, 2.0 * w * q.y);
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) rowsum[j] = red[0];
}

// <a, b> = sum Re(conj a b) per row
__global__ void k_dot_rows(const double2* __restrict__ a, const double2* __restrict__ b, int nh,
                           double* rowsum) {
  const int j = blockIdx.x;
  double acc = 0.0;
  for (int i = threadIdx.x; i < nh; i += blockDim.x) {
    const size_t o = (size_t)j * nh + i;
    acc += a[o].x * b[o].x + a[o].y * b[o].y;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) rowsum[j] = red[0];
}

__global__ void k_sum_in_order(const double* __restrict__ x, int n, double* out) {
  if (threadIdx.x != 0) return;
  double s = 0.0;
  for (int k = 0; k < n; ++k) s += x[k];
  *out = s;
}

// <lam, g> for the unit-amplitude kick g of the LCG state seed0 (forcing.f90:16-33 with famp
// factored out): sdt (cos te, sin te) on each forced mode, sdt (cos te, -sin te) on the
// conjugate partner of the kx=0 and Nyquist modes.
__global__ void k_forcing_dot(const double2* __restrict__ lam, int nh, int nf, const int* __restrict__ ikx,
                              const int* __restrict__ iky, const int* __restrict__ jc,
                              const uint32_t* __restrict__ lcga, const uint32_t* __restrict__ lcgb,
                              uint32_t seed0, double sdt, double* out) {
  const double pi2 = 2.0 * 3.14159265358979;
  double acc = 0.0;
  for (int k = threadIdx.x; k < nf; k += blockDim.x) {
    const uint32_t x = (lcga[k] * seed0 + lcgb[k]) & 0x7FFFFFFFu;
    const float rr = (float)((double)x / 2147483647.0);
    double cs, cc;
    sincos(pi2 * (double)rr, &cs, &cc);
    const int i = ikx[k], j = iky[k];
    const double2 l = lam[(size_t)j * nh + i];
    acc += sdt * (l.x * cc + l.y * cs);
    if (i == 0 || i == nh - 1) {
      const double2 lc = lam[(size_t)jc[j] * nh + i];
      acc += sdt * (lc.x * cc - lc.y * cs);
    }
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// Elementwise parts of the adjoint of one Lawson RK4 step (e = emk, the half-step factor;
// L = the gradient after the step with the (0,0) mode removed, g = the last transposed term):
//   mode 0: L = P0 L (in place), mu = dt/6 L,            acc = e^2 L
//   mode 1: mu = dt e g + dt/3 e L,                      acc += e^2 g
//   mode 2: mu = dt/2 g + dt/3 e L,                      acc += e g
//   mode 3: mu = dt/2 e g + dt/6 e^2 L,                  acc += e g
__global__ void k_adj_rk4_combo(int mode, double2* __restrict__ L, const double2* __restrict__ g,
                                double2* __restrict__ mu, double2* __restrict__ acc,
                                const double* __restrict__ emk, size_t count, double dt) {
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < count;
       o += (size_t)gridDim.x * blockDim.x) {
    const double e = emk[o];
    const double2 l = (mode == 0 && o == 0) ? make_double2(0.0, 0.0) : L[o];
    double cl, cg, ca;  // mu = cg g + cl L; acc (+)= ca (g or L)
    switch (mode) {
      case 0: {
        L[o] = l;
        mu[o] = make_double2(dt / 6.0 * l.x, dt / 6.0 * l.y);
        acc[o] = make_double2(e * e * l.x, e * e * l.y);
        continue;
      }
      case 1: cg = dt * e; cl = dt / 3.0 * e; ca = e * e; break;
      case 2: cg = 0.5 * dt; cl = dt / 3.0 * e; ca = e; break;
      default: cg = 0.5 * dt * e; cl = dt / 6.0 * e * e; ca = e; break;
    }
    const double2 gv = g[o];
    mu[o] = make_double2(fma(cg, gv.x, cl * l.x), fma(cg, gv.y, cl * l.y));
    const double2 av = acc[o];
    acc[o] = make_double2(fma(ca, gv.x, av.x), fma(ca, gv.y, av.y));
  }
}

// Stage k of the Lawson RK4 step and of its tangent (the arithmetic of the epilogues
// EPI_RK4A..D of the forward passes, applied to the state and to the tangent): n, dn = N and dN
// at the stage input; z, dz the step's state (overwritten by k = 3); zn, dzn the accumulated
// znew; w, dw the next stage input (k = 0..2).
__global__ void k_tlm_rk4_update(int k, const double2* __restrict__ n, const double2* __restrict__ dn,
                                 double2* __restrict__ z, double2* __restrict__ dz, double2* __restrict__ zn,
                                 double2* __restrict__ dzn, double2* __restrict__ w, double2* __restrict__ dw,
                                 const double* __restrict__ emk, size_t count, double dt, double dt2,
                                 double dt3, double dt6) {
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < count;
       o += (size_t)gridDim.x * blockDim.x) {
    const double e = emk[o];
    const double2 a = n[o], da = dn[o];
    if (k == 0) {
      const double ee = e * e;
      const double2 x = z[o], dx = dz[o];
      zn[o] = make_double2(ee * (x.x + dt6 * a.x), ee * (x.y + dt6 * a.y));
      dzn[o] = make_double2(ee * (dx.x + dt6 * da.x), ee * (dx.y + dt6 * da.y));
      w[o] = make_double2(e * (x.x + dt2 * a.x), e * (x.y + dt2 * a.y));
      dw[o] = make_double2(e * (dx.x + dt2 * da.x), e * (dx.y + dt2 * da.y));
    } else if (k < 3) {
      const double d3 = dt3 * e;
      const double2 x = z[o], dx = dz[o], zz = zn[o], dzz = dzn[o];
      zn[o] = make_double2(zz.x + d3 * a.x, zz.y + d3 * a.y);
      dzn[o] = make_double2(dzz.x + d3 * da.x, dzz.y + d3 * da.y);
      if (k == 1) {
        w[o] = make_double2(e * x.x + dt2 * a.x, e * x.y + dt2 * a.y);
        dw[o] = make_double2(e * dx.x + dt2 * da.x, e * dx.y + dt2 * da.y);
      } else {
        w[o] = make_double2(e * (e * x.x + dt * a.x), e * (e * x.y + dt * a.y));
        dw[o] = make_double2(e * (e * dx.x + dt * da.x), e * (e * dx.y + dt * da.y));
      }
    } else {
      const double2 zz = zn[o], dzz = dzn[o];
      z[o] = o == 0 ? make_double2(0.0, 0.0) : make_double2(zz.x + dt6 * a.x, zz.y + dt6 * a.y);
      dz[o] = o == 0 ? make_double2(0.0, 0.0) : make_double2(dzz.x + dt6 * da.x, dzz.y + dt6 * da.y);
    }
  }
}

}  // namespace gt

namespace {

int afail(gt_handle* h, int code, const std::string& msg) { return gt::set_error(h, code, msg.c_str()); }

int acuda(gt_handle* h, cudaError_t e, const char* what) {
  return afail(h, GT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define GA_CUDA(h, call)                                 \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return acuda(h, e_, #call);   \
  } while (0)

// grid size within the adjoint kernels' range (RK2 and RK4)
int check_adj_size(gt_handle* h) {
  if (!h) return afail(nullptr, GT_ERR_ARG, "null handle");
  const gt_params* p = gt::handle_params(h);
  if (p->n > GT_ADJ_MAX_N) return afail(h, GT_ERR_ARG, "adjoint / tangent-linear: n must be <= GT_ADJ_MAX_N (4096)");
  if (p->ny != p->n) return afail(h, GT_ERR_ARG, "adjoint / tangent-linear: square grids only");
  return GT_OK;
}

// the RK2-only entry points (tangent-linear model and the single-step adjoint calls)
int check_adj(gt_handle* h) {
  const int rc = check_adj_size(h);
  if (rc) return rc;
  if (gt::handle_rko(h) != 2) return afail(h, GT_ERR_ARG, "adjoint / tangent-linear: RK2 only");
  return GT_OK;
}

gt::GtOp op_of(const gt_handle* h, int kind) {
  gt::GtOp op;
  std::memset(&op, 0, sizeof(op));
  op.kind = kind;
  op.variant = gt::handle_variant(h);
  op.row_variant = gt::handle_row_variant(h);
  op.stream = gt::handle_stream(h);
  op.pdl = gt::handle_pdl(h);
  op.cluster = gt::handle_col_cluster(h);
  const gt::NltArgs base = gt::handle_nlt_args(h, nullptr, nullptr, nullptr, nullptr, nullptr);
  op.tw = base.tw;
  op.twr = base.twr;
  op.nh = base.nh;
  op.nrows = gt::handle_params(h)->ny;
  return op;
}

// The three passes of one evaluation from kind k0 (pass A, B, C). The forward passes take the
// field-split column kernels where the handle runs them; their q buffer (work[0]) never
// aliases the input here.
int run3(gt_handle* h, gt::GtOp op, int k0) {
  const bool fwd = k0 == gt::OP_NLT_COLINV && gt::handle_col_split(h) &&
                   static_cast<const void*>(op.nlt.zin) != static_cast<const void*>(op.nlt.q);
  // the transposed passes likewise (their inputs x and lin never alias the scratch outputs)
  const bool adj = k0 == gt::OP_ADJ_COLINV && gt::handle_col_split(h);
  const bool tlm = k0 == gt::OP_TLM_COLINV && gt::handle_col_split(h);
  for (int k = 0; k < 3; ++k) {
    op.kind = k0 + k;
    if (fwd && k == 0) op.kind = gt::OP_NLT_COLINV_FS;
    if (fwd && k == 2) op.kind = gt::OP_NLT_COLFWD_FS;
    if (adj && k == 0) op.kind = gt::OP_ADJ_COLINV_FS;
    if (adj && k == 2) op.kind = gt::OP_ADJ_COLFWD_FS;
    if (tlm && k == 0) op.kind = gt::OP_TLM_COLINV_FS;
    if (tlm && k == 2) op.kind = gt::OP_TLM_COLFWD_FS;
    const cudaError_t e = gt::handle_dispatch(h, op);
    if (e != cudaSuccess) return acuda(h, e, "adjoint launch");
  }
  return GT_OK;
}

size_t field_bytes(const gt_handle* h) {
  const int n = gt::handle_params(h)->n;
  return sizeof(double) * (size_t)(n + 2) * n;
}

// objective into d_out (device double), gradient into grad (device, may be null)
int objective_dev(gt_handle* h, const double* z, double kmin, double kmax, double* grad,
                  double* d_rows, double* d_out) {
  const gt_params* p = gt::handle_params(h);
  const int n = p->n, nh = n / 2 + 1;
  const double *fkxs, *fkys;
  gt::handle_k2(h, &fkxs, &fkys);
  const gt::NltArgs t = gt::handle_nlt_args(h, nullptr, nullptr, nullptr, nullptr, nullptr);
  cudaStream_t s = gt::handle_stream(h);
  gt::k_objective_rows<<<n, 256, 0, s>>>(reinterpret_cast<const double2*>(z), fkxs, fkys, t.kainv, nh,
                                         kmin * kmin, kmax * kmax, d_rows, reinterpret_cast<double2*>(grad));
  gt::k_sum_in_order<<<1, 32, 0, s>>>(d_rows, n, d_out);
  GA_CUDA(h, cudaGetLastError());
  return GT_OK;
}

int forcing_dot_dev(gt_handle* h, const double* lam, uint32_t seed0, double* d_out) {
  const gt::ForcingView f = gt::handle_forcing(h);
  if (f.nf == 0) {
    GA_CUDA(h, cudaMemsetAsync(d_out, 0, sizeof(double), gt::handle_stream(h)));
    return GT_OK;
  }
  gt::k_forcing_dot<<<1, 256, 0, gt::handle_stream(h)>>>(reinterpret_cast<const double2*>(lam), f.nh, f.nf,
                                                         f.ikx, f.iky, f.jc, f.lcga, f.lcgb, seed0, f.sdt, d_out);
  GA_CUDA(h, cudaGetLastError());
  return GT_OK;
}

// Physical fields of one forward evaluation, as its pass B stores them (both null: not kept).
struct Phys {
  double2* uv = nullptr;
  double2* q = nullptr;
};

// Segments the forward sweep of gt_adj_gradient keeps whole: as many of its last segments as
// the handle's budget (gt_adj_set_memory) holds, at least one (the storage a recomputed segment
// needs anyway) and at most all of them; never more than 90 % of the free device memory allows.
// step_bytes: one step's stage states and physical fields.
int kept_segments(const gt_handle* h, int ncp, int K, size_t step_bytes) {
  const int64_t seg = (int64_t)K * (int64_t)step_bytes;
  int64_t budget = gt::handle_adj_memory(h);
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
    const int64_t cap = (int64_t)(0.9 * (double)free_b);
    if (budget > cap) budget = cap;
  } else {
    cudaGetLastError();
  }
  const int64_t fit = seg > 0 ? budget / seg : 0;
  return (int)std::max<int64_t>(1, std::min<int64_t>(ncp, fit));
}

// w = P0 e (z + dt/2 N(z)): the forward stage A with the fused passes (work: 3 fields)
int stage_a(gt_handle* h, const double* z, double* w, double* const* work, Phys keep = Phys()) {
  gt::GtOp op = op_of(h, gt::OP_NLT_COLINV);
  op.nlt = gt::handle_nlt_args(h, z, work[0], work[1], work[2], gt::handle_flag(h));
  op.nlt.phys_uv = keep.uv;
  op.nlt.phys_q = keep.q;
  op.nlt.epi.mode = gt::EPI_RK2A;
  op.nlt.epi.out = reinterpret_cast<double2*>(w);
  op.nlt.epi.z = reinterpret_cast<const double2*>(z);
  return run3(h, op, gt::OP_NLT_COLINV);
}

// z_next = P0 e (e z + dt N(w)) written to `out` (may alias z) (work: 3 fields)
int stage_b(gt_handle* h, const double* w, double* out, double* const* work, Phys keep = Phys()) {
  gt::GtOp op = op_of(h, gt::OP_NLT_COLINV);
  op.nlt = gt::handle_nlt_args(h, w, work[0], work[1], work[2], gt::handle_flag(h));
  op.nlt.phys_uv = keep.uv;
  op.nlt.phys_q = keep.q;
  op.nlt.epi.mode = gt::EPI_RK2B;
  op.nlt.epi.out = reinterpret_cast<double2*>(out);
  op.nlt.epi.z = reinterpret_cast<const double2*>(out);
  return run3(h, op, gt::OP_NLT_COLINV);
}

gt::TlmArgs tlm_args(const gt_handle* h) {
  const gt::NltArgs t = gt::handle_nlt_args(h, nullptr, nullptr, nullptr, nullptr, nullptr);
  gt::TlmArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n = t.n;
  a.kainv = t.kainv;
  a.fkx = t.fkx;
  a.fky = t.fky;
  a.kcut = t.kcut;
  a.tw = t.tw;
  a.truncate = t.truncate;
  a.emk = t.epi.emk;
  a.emkx = t.epi.emkx;
  a.emky = t.epi.emky;
  a.split = t.epi.split;
  a.dt = t.epi.dt;
  a.dt2 = t.epi.dt2;
  a.colcnt = t.colcnt;
  return a;
}

gt::AdjArgs adj_args(const gt_handle* h) {
  const gt::TlmArgs t = tlm_args(h);
  gt::AdjArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n = t.n;
  a.kainv = t.kainv;
  a.fkx = t.fkx;
  a.fky = t.fky;
  a.kcut = t.kcut;
  a.tw = t.tw;
  a.truncate = t.truncate;
  a.emk = t.emk;
  a.emkx = t.emkx;
  a.emky = t.emky;
  a.split = t.split;
  a.dt = t.dt;
  a.dt2 = t.dt2;
  const gt::NltArgs nl = gt::handle_nlt_args(h, nullptr, nullptr, nullptr, nullptr, nullptr);
  a.kxlim = nl.kxlim;
  a.colcnt = nl.colcnt;
  return a;
}

// lam = dF(x)^T lin (mode ADJ_PLAIN) or lam += dF(x)^T lin (ADJ_STAGE_A); work: q, u, v, a, b
int adj_term(gt_handle* h, int mode, const double* x, const double* lin, double* lam, double* const* work,
             Phys px = Phys()) {
  gt::GtOp op = op_of(h, gt::OP_ADJ_COLINV);
  gt::AdjArgs a = adj_args(h);
  a.phys_uv = px.uv;  // the physical fields of the forward evaluation at x, when kept
  a.phys_q = px.q;
  a.q = reinterpret_cast<double2*>(work[0]);
  a.u = reinterpret_cast<double2*>(work[1]);
  a.v = reinterpret_cast<double2*>(work[2]);
  a.a = reinterpret_cast<double2*>(work[3]);
  a.b = reinterpret_cast<double2*>(work[4]);
  a.mode = mode;
  a.x = reinterpret_cast<const double2*>(x);
  a.lin = reinterpret_cast<const double2*>(lin);
  a.lam = reinterpret_cast<double2*>(lam);
  op.adj = a;
  return run3(h, op, gt::OP_ADJ_COLINV);
}

// one adjoint step (without the forcing dot), work: q, u, v, a, b, rho; pz, pw: the physical
// fields of the forward evaluations at z and w when the caller kept them
int adj_step(gt_handle* h, const double* z, const double* w, double* lam, double* const* work,
             Phys pz = Phys(), Phys pw = Phys()) {
  gt::GtOp op = op_of(h, gt::OP_ADJ_COLINV);
  gt::AdjArgs a = adj_args(h);
  a.q = reinterpret_cast<double2*>(work[0]);
  a.u = reinterpret_cast<double2*>(work[1]);
  a.v = reinterpret_cast<double2*>(work[2]);
  a.a = reinterpret_cast<double2*>(work[3]);
  a.b = reinterpret_cast<double2*>(work[4]);
  a.rho = reinterpret_cast<double2*>(work[5]);
  a.lam = reinterpret_cast<double2*>(lam);
  // second half of the step: linearised at w, input l'
  a.mode = gt::ADJ_STAGE_B;
  a.x = reinterpret_cast<const double2*>(w);
  a.lin = reinterpret_cast<const double2*>(lam);
  a.phys_uv = pw.uv;
  a.phys_q = pw.q;
  op.adj = a;
  int rc = run3(h, op, gt::OP_ADJ_COLINV);
  if (rc) return rc;
  // first half: linearised at z, input rho
  a.mode = gt::ADJ_STAGE_A;
  a.x = reinterpret_cast<const double2*>(z);
  a.lin = a.rho;
  a.phys_uv = pz.uv;
  a.phys_q = pz.q;
  op.adj = a;
  return run3(h, op, gt::OP_ADJ_COLINV);
}

// Stage k (0..3) of the Lawson RK4 step from z (src/rkstep.f90:91-128, the fused passes with
// epilogues EPI_RK4A..D): evaluates N at zin (z, w1, w2, w3), writes the next stage state (w1,
// w2, w3, or the new state for k = 3) to out and accumulates znew. work: q, u, v scratch
// distinct from zin, out and z.
int rk4_stage(gt_handle* h, int k, const double* z, const double* zin, double* out, double* znew,
              double* const* work, Phys keep = Phys()) {
  gt::GtOp op = op_of(h, gt::OP_NLT_COLINV);
  op.nlt = gt::handle_nlt_args(h, zin, work[0], work[1], work[2], gt::handle_flag(h));
  op.nlt.phys_uv = keep.uv;
  op.nlt.phys_q = keep.q;
  op.nlt.epi.mode = gt::EPI_RK4A + k;
  op.nlt.epi.out = reinterpret_cast<double2*>(out);
  op.nlt.epi.znew = reinterpret_cast<double2*>(znew);
  op.nlt.epi.z = reinterpret_cast<const double2*>(z);
  return run3(h, op, gt::OP_NLT_COLINV);
}

// One RK4 step of z in place keeping its stage states w1, w2, w3 (work: q, u, v scratch).
// keep: the physical fields of the evaluations at z, w1, w2, w3 (null entries: not kept).
int rk4_step_keep(gt_handle* h, double* z, double* w1, double* w2, double* w3, double* znew,
                  double* const* work, const Phys* keep = nullptr) {
  const Phys none;
  auto kp = [&](int k) { return keep ? keep[k] : none; };
  int rc = rk4_stage(h, 0, z, z, w1, znew, work, kp(0));
  if (!rc) rc = rk4_stage(h, 1, z, w1, w2, znew, work, kp(1));
  if (!rc) rc = rk4_stage(h, 2, z, w2, w3, znew, work, kp(2));
  if (!rc) rc = rk4_stage(h, 3, z, w3, z, znew, work, kp(3));  // stage D reads znew, not z
  return rc;
}

// Adjoint of one Lawson RK4 step (stage states z, w1, w2, w3 of the step; the forcing kick is
// additive and its adjoint is the identity): lam = dJ/d(state after the step) on entry, dJ/dz on
// return. With L = P0 lam (the step's last stage zeroes the (0,0) mode):
//   mu4 = dt/6 L                   g4 = dF(w3)^T mu4
//   mu3 = dt e g4 + dt/3 e L        g3 = dF(w2)^T mu3
//   mu2 = dt/2 g3 + dt/3 e L        g2 = dF(w1)^T mu2
//   mu1 = dt/2 e g2 + dt/6 e^2 L    g1 = dF(z)^T mu1
//   dJ/dz = e^2 L + e^2 g4 + e g3 + e g2 + g1
// work: q, u, v, a, b, g, mu, acc (8 fields).
int adj_step_rk4(gt_handle* h, const double* z, const double* w1, const double* w2, const double* w3,
                 double* lam, double* const* work, const Phys* keep = nullptr) {
  const Phys none;
  auto kp = [&](int k) { return keep ? keep[k] : none; };  // at z, w1, w2, w3
  const gt_params* p = gt::handle_params(h);
  const int n = p->n, nh = n / 2 + 1;
  const size_t count = (size_t)n * nh;
  double2* L = reinterpret_cast<double2*>(lam);
  double2* g = reinterpret_cast<double2*>(work[5]);
  double2* mu = reinterpret_cast<double2*>(work[6]);
  double2* acc = reinterpret_cast<double2*>(work[7]);
  const double* emk = gt::handle_nlt_args(h, nullptr, nullptr, nullptr, nullptr, nullptr).epi.emk;
  cudaStream_t s = gt::handle_stream(h);
  const int blocks = (int)((count + 255) / 256 < 4 * 152 ? (count + 255) / 256 : 4 * 152);
  auto combo = [&](int mode) {
    gt::k_adj_rk4_combo<<<blocks, 256, 0, s>>>(mode, L, g, mu, acc, emk, count, p->dt);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GT_OK : acuda(h, e, "adjoint RK4 update");
  };
  const double* ws[3] = {w3, w2, w1};
  int rc = combo(0);
  for (int k = 0; k < 3 && !rc; ++k) {
    rc = adj_term(h, gt::ADJ_PLAIN, ws[k], work[6], work[5], work, kp(3 - k));
    if (!rc) rc = combo(k + 1);
  }
  if (!rc) rc = adj_term(h, gt::ADJ_STAGE_A, z, work[6], work[7], work, kp(0));
  if (rc) return rc;
  GA_CUDA(h, cudaMemcpyAsync(lam, work[7], sizeof(double2) * count, cudaMemcpyDeviceToDevice, s));
  return GT_OK;
}

// One tangent-linear RK4 step + kick: z advances as gt_step_rk4 + gt_forcing(z, seed), dz by the
// derivative of that step plus dfamp times the kick of the same draws. work: q, u, v, dq, du, dv,
// znew, dznew, w, dw (10 fields).
int tlm_step_rk4(gt_handle* h, double* z, double* dz, double dfamp, int32_t* seed, double* const* work) {
  const gt::NltArgs t = gt::handle_nlt_args(h, nullptr, nullptr, nullptr, nullptr, nullptr);
  const int n = t.n;
  const size_t count = (size_t)n * (n / 2 + 1);
  cudaStream_t s = gt::handle_stream(h);
  const int blocks = (int)((count + 255) / 256 < 4 * 152 ? (count + 255) / 256 : 4 * 152);
  auto F = [&](int k) { return reinterpret_cast<double2*>(work[k]); };
  gt::GtOp op = op_of(h, gt::OP_TLM_COLINV);
  gt::TlmArgs a = tlm_args(h);
  a.q = F(0); a.u = F(1); a.v = F(2); a.dq = F(3); a.du = F(4); a.dv = F(5);
  a.mode = gt::TLM_PLAIN;
  double2* zz = reinterpret_cast<double2*>(z);
  double2* dzz = reinterpret_cast<double2*>(dz);
  for (int k = 0; k < 4; ++k) {
    a.x = k == 0 ? zz : F(8);
    a.dx = k == 0 ? dzz : F(9);
    op.tlm = a;
    int rc = run3(h, op, gt::OP_TLM_COLINV);
    if (rc) return rc;
    // the next stage input goes to (w, dw) = work 8, 9: stage k reads them, so stage k writes
    // its update after its own passes (N, dN are already in u, du)
    gt::k_tlm_rk4_update<<<blocks, 256, 0, s>>>(k, F(1), F(4), zz, dzz, F(6), F(7), F(8), F(9),
                                                t.epi.emk, count, t.epi.dt, t.epi.dt2, t.epi.dt3, t.epi.dt6);
    GA_CUDA(h, cudaGetLastError());
  }
  const uint32_t s0 = (uint32_t)(*seed);
  GA_CUDA(h, gt::forcing_amp(h, z, s0, gt::handle_params(h)->famp));
  GA_CUDA(h, gt::forcing_amp(h, dz, s0, dfamp));
  const gt::ForcingView f = gt::handle_forcing(h);
  if (f.nf > 0) *seed = (int32_t)((f.lcga_nf * s0 + f.lcgb_nf) & 0x7FFFFFFFu);
  return GT_OK;
}

struct DevPool {
  std::vector<void*> ptrs;
  ~DevPool() {
    for (void* p : ptrs) cudaFree(p);
  }
  double* field(size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<double*>(p);
  }
};

// gt_adj_gradient for the RK4 integrator: checkpoints every K steps, the last segment kept by
// the forward sweep, each earlier segment recomputed with its stage states (z, w1, w2, w3).
int gradient_rk4(gt_handle* h, const double* z0, int nsteps, int32_t seed, int K, double kmin, double kmax,
                 double* J, double* grad_z0, double* grad_famp, double* zT, double* times_ms) {
  cudaStream_t s = gt::handle_stream(h);
  const size_t fb = field_bytes(h);
  const int n = gt::handle_params(h)->n;
  const int ncp = (nsteps + K - 1) / K;
  const size_t uvb = sizeof(double2) * (size_t)n * n, qb = sizeof(double2) * (size_t)n * (n / 2);
  // the forward sweep keeps its last m segments whole (slots for m K steps)
  const int m = kept_segments(h, ncp, K, 4 * fb + 4 * (uvb + qb));
  const int slots = m * K;
  DevPool pool;
  std::vector<double*> cp(ncp), zs(slots), w1(slots), w2(slots), w3(slots), work(8);
  for (auto* v : {&cp, &zs, &w1, &w2, &w3, &work})
    for (auto& q : *v) q = pool.field(fb);
  double* z = pool.field(fb);
  double* znew = pool.field(fb);
  double* lam = pool.field(fb);
  double* scal = pool.field(sizeof(double) * ((size_t)nsteps + n + 2));
  if (pool.ptrs.size() != (size_t)(ncp + 4 * slots + 8 + 4))
    return afail(h, GT_ERR_NOMEM, "gt_adj_gradient: cudaMalloc of the checkpoint storage failed");
  double* dots = scal;
  double* rows = scal + nsteps;
  // the physical u+iv and q of the 4 stage evaluations of every slot's step (24 N^2 bytes each),
  // read by the transposed terms; without the memory for them those terms transform x themselves
  DevPool phys_pool;
  std::vector<Phys> keep(4 * (size_t)slots);
  {
    bool ok = true;
    for (auto& k : keep) {
      if (!ok) break;
      k.uv = reinterpret_cast<double2*>(phys_pool.field(uvb));
      k.q = reinterpret_cast<double2*>(phys_pool.field(qb));
      ok = k.uv && k.q;
    }
    if (!ok) {
      cudaGetLastError();  // clear the failed allocation
      for (auto& k : keep) k = Phys();
    }
  }
  cudaEvent_t e0, e1, e2;
  GA_CUDA(h, cudaEventCreate(&e0));
  GA_CUDA(h, cudaEventCreate(&e1));
  GA_CUDA(h, cudaEventCreate(&e2));
  std::vector<int32_t> seeds(nsteps);
  GA_CUDA(h, cudaEventRecord(e0, s));
  GA_CUDA(h, cudaMemcpyAsync(z, z0, fb, cudaMemcpyDeviceToDevice, s));
  const int keep0 = (ncp - m) * K;  // first step of the kept segments
  int32_t sd = seed;
  int rc = GT_OK;
  for (int st = 0; st < nsteps; ++st) {
    if (st % K == 0) GA_CUDA(h, cudaMemcpyAsync(cp[st / K], z, fb, cudaMemcpyDeviceToDevice, s));
    seeds[st] = sd;
    const int r = st >= keep0 ? st - keep0 : 0;  // earlier steps use slot 0 as scratch
    if (st >= keep0) GA_CUDA(h, cudaMemcpyAsync(zs[r], z, fb, cudaMemcpyDeviceToDevice, s));
    rc = rk4_step_keep(h, z, w1[r], w2[r], w3[r], znew, work.data(), st >= keep0 ? &keep[4 * (size_t)r] : nullptr);
    if (!rc) rc = gt_forcing(h, z, &sd);
    if (rc) return rc;
  }
  if (zT) GA_CUDA(h, cudaMemcpyAsync(zT, z, fb, cudaMemcpyDeviceToDevice, s));
  rc = objective_dev(h, z, kmin, kmax, lam, rows, rows + n);
  if (rc) return rc;
  GA_CUDA(h, cudaEventRecord(e1, s));
  for (int c = ncp - 1; c >= 0; --c) {
    const int s0 = c * K, s1 = (s0 + K < nsteps) ? s0 + K : nsteps;
    const bool kept = c >= ncp - m;        // stored by the forward sweep
    const int base = kept ? s0 - keep0 : 0;  // its first slot (recomputed segments: slot 0)
    if (!kept) {  // recompute the segment's stage states from its checkpoint
      GA_CUDA(h, cudaMemcpyAsync(zs[0], cp[c], fb, cudaMemcpyDeviceToDevice, s));
      for (int st = s0; st < s1; ++st) {
        const int r = st - s0;
        const Phys* kr = &keep[4 * (size_t)r];
        rc = rk4_stage(h, 0, zs[r], zs[r], w1[r], znew, work.data(), kr[0]);
        if (!rc) rc = rk4_stage(h, 1, zs[r], w1[r], w2[r], znew, work.data(), kr[1]);
        if (!rc) rc = rk4_stage(h, 2, zs[r], w2[r], w3[r], znew, work.data(), kr[2]);
        if (!rc && st + 1 < s1) {
          rc = rk4_stage(h, 3, zs[r], w3[r], zs[r + 1], znew, work.data(), kr[3]);
          int32_t sk = seeds[st];
          if (!rc) rc = gt_forcing(h, zs[r + 1], &sk);
        }
        if (rc) return rc;
      }
    }
    for (int st = s1 - 1; st >= s0; --st) {
      const int r = base + st - s0;
      rc = forcing_dot_dev(h, lam, (uint32_t)seeds[st], dots + st);
      // a recomputed segment's last stage D was not evaluated: its term transforms w3 itself
      Phys kr[4] = {keep[4 * (size_t)r], keep[4 * (size_t)r + 1], keep[4 * (size_t)r + 2], keep[4 * (size_t)r + 3]};
      if (!kept && st + 1 == s1) kr[3] = Phys();
      if (!rc) rc = adj_step_rk4(h, zs[r], w1[r], w2[r], w3[r], lam, work.data(), kr);
      if (rc) return rc;
    }
  }
  GA_CUDA(h, cudaEventRecord(e2, s));
  GA_CUDA(h, cudaMemcpyAsync(grad_z0, lam, fb, cudaMemcpyDeviceToDevice, s));
  std::vector<double> host(nsteps + 1);
  GA_CUDA(h, cudaMemcpyAsync(host.data(), dots, sizeof(double) * nsteps, cudaMemcpyDeviceToHost, s));
  GA_CUDA(h, cudaMemcpyAsync(host.data() + nsteps, rows + n, sizeof(double), cudaMemcpyDeviceToHost, s));
  GA_CUDA(h, cudaStreamSynchronize(s));
  *J = host[nsteps];
  if (grad_famp) {
    double g = 0.0;
    for (int st = 0; st < nsteps; ++st) g += host[st];
    *grad_famp = g;
  }
  if (times_ms) {
    float f = 0.f, b = 0.f;
    cudaEventElapsedTime(&f, e0, e1);
    cudaEventElapsedTime(&b, e1, e2);
    times_ms[0] = f;
    times_ms[1] = b;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  return GT_OK;
}

}  // namespace

extern "C" {

int gt_objective(gt_handle* h, const double* z, double kmin, double kmax, double* J, double* grad) {
  if (!h || !z || !J) return afail(h, GT_ERR_ARG, "gt_objective: null argument");
  if (gt::handle_params(h)->ny != gt::handle_params(h)->n)
    return afail(h, GT_ERR_ARG, "gt_objective: square grids only");
  DevPool pool;
  const int n = gt::handle_params(h)->n;
  double* rows = pool.field(sizeof(double) * (n + 1));
  if (!rows) return afail(h, GT_ERR_NOMEM, "gt_objective: cudaMalloc");
  int rc = objective_dev(h, z, kmin, kmax, grad, rows, rows + n);
  if (rc) return rc;
  GA_CUDA(h, cudaMemcpyAsync(J, rows + n, sizeof(double), cudaMemcpyDeviceToHost, gt::handle_stream(h)));
  GA_CUDA(h, cudaStreamSynchronize(gt::handle_stream(h)));
  return GT_OK;
}

int gt_tlm_step_rk2(gt_handle* h, double* z, double* dz, double dfamp, int32_t* seed, double* const* work) {
  int rc = check_adj(h);
  if (rc) return rc;
  if (!z || !dz || !seed || !work) return afail(h, GT_ERR_ARG, "gt_tlm_step_rk2: null argument");
  for (int k = 0; k < 8; ++k)
    if (!work[k]) return afail(h, GT_ERR_ARG, "gt_tlm_step_rk2: null work field");
  gt::GtOp op = op_of(h, gt::OP_TLM_COLINV);
  gt::TlmArgs a = tlm_args(h);
  a.q = reinterpret_cast<double2*>(work[2]);
  a.u = reinterpret_cast<double2*>(work[3]);
  a.v = reinterpret_cast<double2*>(work[4]);
  a.dq = reinterpret_cast<double2*>(work[5]);
  a.du = reinterpret_cast<double2*>(work[6]);
  a.dv = reinterpret_cast<double2*>(work[7]);
  a.z = reinterpret_cast<double2*>(z);
  a.dz = reinterpret_cast<double2*>(dz);
  a.w = reinterpret_cast<double2*>(work[0]);
  a.dw = reinterpret_cast<double2*>(work[1]);
  a.mode = gt::TLM_STAGE_A;
  a.x = a.z;
  a.dx = a.dz;
  op.tlm = a;
  rc = run3(h, op, gt::OP_TLM_COLINV);
  if (rc) return rc;
  a.mode = gt::TLM_STAGE_B;
  a.x = a.w;
  a.dx = a.dw;
  op.tlm = a;
  rc = run3(h, op, gt::OP_TLM_COLINV);
  if (rc) return rc;
  const uint32_t s0 = (uint32_t)(*seed);
  GA_CUDA(h, gt::forcing_amp(h, z, s0, gt::handle_params(h)->famp));
  GA_CUDA(h, gt::forcing_amp(h, dz, s0, dfamp));
  const gt::ForcingView f = gt::handle_forcing(h);
  if (f.nf > 0) *seed = (int32_t)((f.lcga_nf * s0 + f.lcgb_nf) & 0x7FFFFFFFu);
  return GT_OK;
}

int gt_adj_stage(gt_handle* h, const double* z, double* w, double* const* work) {
  int rc = check_adj(h);
  if (rc) return rc;
  if (!z || !w || !work || !work[0] || !work[1] || !work[2]) return afail(h, GT_ERR_ARG, "gt_adj_stage: null argument");
  return stage_a(h, z, w, work);
}

int gt_adj_step_rk2(gt_handle* h, const double* z, const double* w, double* lam, int32_t seed,
                    double* gfamp, double* const* work) {
  int rc = check_adj(h);
  if (rc) return rc;
  if (!z || !w || !lam || !work) return afail(h, GT_ERR_ARG, "gt_adj_step_rk2: null argument");
  for (int k = 0; k < 6; ++k)
    if (!work[k]) return afail(h, GT_ERR_ARG, "gt_adj_step_rk2: null work field");
  if (gfamp) {
    DevPool pool;
    double* d = pool.field(sizeof(double));
    if (!d) return afail(h, GT_ERR_NOMEM, "gt_adj_step_rk2: cudaMalloc");
    rc = forcing_dot_dev(h, lam, (uint32_t)seed, d);
    if (rc) return rc;
    double v = 0.0;
    GA_CUDA(h, cudaMemcpyAsync(&v, d, sizeof(double), cudaMemcpyDeviceToHost, gt::handle_stream(h)));
    GA_CUDA(h, cudaStreamSynchronize(gt::handle_stream(h)));
    *gfamp += v;
  }
  return adj_step(h, z, w, lam, work);
}

int gt_adj_gradient(gt_handle* h, const double* z0, int32_t nsteps, int32_t seed, int32_t K, double kmin,
                    double kmax, double* J, double* grad_z0, double* grad_famp, double* zT, double* times_ms) {
  int rc = check_adj_size(h);
  if (rc) return rc;
  if (!z0 || !J || !grad_z0 || nsteps < 1 || K < 1) return afail(h, GT_ERR_ARG, "gt_adj_gradient: bad argument");
  if (gt::handle_rko(h) == 4)
    return gradient_rk4(h, z0, nsteps, seed, K, kmin, kmax, J, grad_z0, grad_famp, zT, times_ms);
  cudaStream_t s = gt::handle_stream(h);
  const size_t fb = field_bytes(h);
  const int n = gt::handle_params(h)->n;
  const int ncp = (nsteps + K - 1) / K;
  const size_t uvb = sizeof(double2) * (size_t)n * n, qb = sizeof(double2) * (size_t)n * (n / 2);
  // the forward sweep keeps its last m segments whole (slots for m K steps)
  const int m = kept_segments(h, ncp, K, 2 * fb + 2 * (uvb + qb));
  const int slots = m * K;
  DevPool pool;
  std::vector<double*> cp(ncp), zs(slots), ws(slots), work(6);
  for (auto& p : cp) p = pool.field(fb);
  for (auto& p : zs) p = pool.field(fb);
  for (auto& p : ws) p = pool.field(fb);
  for (auto& p : work) p = pool.field(fb);
  double* z = pool.field(fb);
  double* lam = pool.field(fb);
  double* scal = pool.field(sizeof(double) * ((size_t)nsteps + n + 2));
  if (pool.ptrs.size() != (size_t)(ncp + 2 * slots + 6 + 3))
    return afail(h, GT_ERR_NOMEM, "gt_adj_gradient: cudaMalloc of the checkpoint storage failed");
  double* dots = scal;           // [nsteps]
  double* rows = scal + nsteps;  // [n + 1], objective scratch + result
  // The physical u+iv and q of both stages of every slot's step (24 N^2 bytes each), so that the
  // adjoint passes do not transform the linearisation points again. Without the memory for them
  // the adjoint recomputes those transforms itself.
  DevPool phys_pool;
  std::vector<Phys> pz(slots), pw(slots);
  {
    bool ok = true;
    for (int r = 0; r < slots && ok; ++r) {
      pz[r].uv = reinterpret_cast<double2*>(phys_pool.field(uvb));
      pz[r].q = reinterpret_cast<double2*>(phys_pool.field(qb));
      pw[r].uv = reinterpret_cast<double2*>(phys_pool.field(uvb));
      pw[r].q = reinterpret_cast<double2*>(phys_pool.field(qb));
      ok = pz[r].uv && pz[r].q && pw[r].uv && pw[r].q;
    }
    if (!ok) {
      cudaGetLastError();  // clear the failed allocation
      for (int r = 0; r < slots; ++r) pz[r] = pw[r] = Phys();
    }
  }
  cudaEvent_t e0, e1, e2;
  GA_CUDA(h, cudaEventCreate(&e0));
  GA_CUDA(h, cudaEventCreate(&e1));
  GA_CUDA(h, cudaEventCreate(&e2));
  std::vector<int32_t> seeds(nsteps);
  GA_CUDA(h, cudaEventRecord(e0, s));
  // forward sweep, checkpoint every K steps
  GA_CUDA(h, cudaMemcpyAsync(z, z0, fb, cudaMemcpyDeviceToDevice, s));
  // The last m segments keep their states (z_s, w_s) and physical fields as they go: the
  // backward sweep runs over them without recomputing them.
  const int keep0 = (ncp - m) * K;
  int32_t sd = seed;
  for (int st = 0; st < nsteps; ++st) {
    if (st % K == 0) GA_CUDA(h, cudaMemcpyAsync(cp[st / K], z, fb, cudaMemcpyDeviceToDevice, s));
    seeds[st] = sd;
    if (st >= keep0) {
      const int r = st - keep0;
      GA_CUDA(h, cudaMemcpyAsync(zs[r], z, fb, cudaMemcpyDeviceToDevice, s));
      rc = stage_a(h, z, ws[r], work.data(), pz[r]);
      if (!rc) rc = stage_b(h, ws[r], z, work.data(), pw[r]);
    } else {
      rc = stage_a(h, z, ws[0], work.data());
      if (!rc) rc = stage_b(h, ws[0], z, work.data());
    }
    if (!rc) rc = gt_forcing(h, z, &sd);
    if (rc) return rc;
  }
  if (zT) GA_CUDA(h, cudaMemcpyAsync(zT, z, fb, cudaMemcpyDeviceToDevice, s));
  rc = objective_dev(h, z, kmin, kmax, lam, rows, rows + n);
  if (rc) return rc;
  GA_CUDA(h, cudaEventRecord(e1, s));
  // backward sweep: per segment, recompute and store (z_s, w_s), then run the adjoint back
  for (int c = ncp - 1; c >= 0; --c) {
    const int s0 = c * K, s1 = (s0 + K < nsteps) ? s0 + K : nsteps;
    const bool kept = c >= ncp - m;          // stored by the forward sweep
    const int base = kept ? s0 - keep0 : 0;  // its first slot (recomputed segments: slot 0)
    if (!kept) GA_CUDA(h, cudaMemcpyAsync(zs[0], cp[c], fb, cudaMemcpyDeviceToDevice, s));
    for (int st = s0; st < s1 && !kept; ++st) {
      const int r = st - s0;
      rc = stage_a(h, zs[r], ws[r], work.data(), pz[r]);
      if (rc) return rc;
      if (st + 1 < s1) {
        GA_CUDA(h, cudaMemcpyAsync(zs[r + 1], zs[r], fb, cudaMemcpyDeviceToDevice, s));
        rc = stage_b(h, ws[r], zs[r + 1], work.data(), pw[r]);
        int32_t sk = seeds[st];
        if (!rc) rc = gt_forcing(h, zs[r + 1], &sk);
        if (rc) return rc;
      }
    }
    for (int st = s1 - 1; st >= s0; --st) {
      const int r = base + st - s0;
      rc = forcing_dot_dev(h, lam, (uint32_t)seeds[st], dots + st);
      // a recomputed segment's last stage B was not evaluated: its adjoint transforms w itself
      if (!rc) rc = adj_step(h, zs[r], ws[r], lam, work.data(), pz[r], (kept || st + 1 < s1) ? pw[r] : Phys());
      if (rc) return rc;
    }
  }
  GA_CUDA(h, cudaEventRecord(e2, s));
  GA_CUDA(h, cudaMemcpyAsync(grad_z0, lam, fb, cudaMemcpyDeviceToDevice, s));
  std::vector<double> host(nsteps + 1);
  GA_CUDA(h, cudaMemcpyAsync(host.data(), dots, sizeof(double) * nsteps, cudaMemcpyDeviceToHost, s));
  GA_CUDA(h, cudaMemcpyAsync(host.data() + nsteps, rows + n, sizeof(double), cudaMemcpyDeviceToHost, s));
  GA_CUDA(h, cudaStreamSynchronize(s));
  *J = host[nsteps];
  if (grad_famp) {
    double g = 0.0;
    for (int st = 0; st < nsteps; ++st) g += host[st];
    *grad_famp = g;
  }
  if (times_ms) {
    float f = 0.f, b = 0.f;
    cudaEventElapsedTime(&f, e0, e1);
    cudaEventElapsedTime(&b, e1, e2);
    times_ms[0] = f;
    times_ms[1] = b;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  return GT_OK;
}

int gt_tlm_run(gt_handle* h, const double* z0, const double* dz0, double dfamp, int32_t nsteps, int32_t seed,
               double kmin, double kmax, double* J, double* dJ) {
  int rc = check_adj_size(h);
  if (rc) return rc;
  if (!z0 || !dz0 || !J || !dJ || nsteps < 0) return afail(h, GT_ERR_ARG, "gt_tlm_run: bad argument");
  cudaStream_t s = gt::handle_stream(h);
  const size_t fb = field_bytes(h);
  const int n = gt::handle_params(h)->n;
  DevPool pool;
  double* z = pool.field(fb);
  double* dz = pool.field(fb);
  double* grad = pool.field(fb);
  const bool rk4 = gt::handle_rko(h) == 4;
  std::vector<double*> work(rk4 ? 10 : 8);
  for (auto& p : work) p = pool.field(fb);
  double* rows = pool.field(sizeof(double) * (2 * (size_t)n + 2));
  if (pool.ptrs.size() != work.size() + 4) return afail(h, GT_ERR_NOMEM, "gt_tlm_run: cudaMalloc failed");
  GA_CUDA(h, cudaMemcpyAsync(z, z0, fb, cudaMemcpyDeviceToDevice, s));
  GA_CUDA(h, cudaMemcpyAsync(dz, dz0, fb, cudaMemcpyDeviceToDevice, s));
  int32_t sd = seed;
  for (int st = 0; st < nsteps; ++st) {
    rc = rk4 ? tlm_step_rk4(h, z, dz, dfamp, &sd, work.data()) : gt_tlm_step_rk2(h, z, dz, dfamp, &sd, work.data());
    if (rc) return rc;
  }
  rc = objective_dev(h, z, kmin, kmax, grad, rows, rows + n);
  if (rc) return rc;
  gt::k_dot_rows<<<n, 256, 0, s>>>(reinterpret_cast<const double2*>(grad), reinterpret_cast<const double2*>(dz),
                                   n / 2 + 1, rows + n + 1);
  gt::k_sum_in_order<<<1, 32, 0, s>>>(rows + n + 1, n, rows + 2 * n + 1);
  GA_CUDA(h, cudaGetLastError());
  double out[2];
  GA_CUDA(h, cudaMemcpyAsync(&out[0], rows + n, sizeof(double), cudaMemcpyDeviceToHost, s));
  GA_CUDA(h, cudaMemcpyAsync(&out[1], rows + 2 * n + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
  GA_CUDA(h, cudaStreamSynchronize(s));
  *J = out[0];
  *dJ = out[1];
  return GT_OK;
}

}  // extern "C"
