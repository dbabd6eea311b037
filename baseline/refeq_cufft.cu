// refeq_cufft.cu -- "reference-equivalent" GPU build of the Gturbo time step.
//
// MEASUREMENT BASELINE ONLY (not part of the product library). The reference is Fortran +
// OpenACC + cuFFT and cannot be compiled here (no nvfortran); this file restates its device
// work launch for launch so that its GPU speed can be measured on the same GB300:
//   nlt.f90:17-20   u=0, v=0                       -> 2 x cudaMemsetAsync
//   nlt.f90:22-36   u_hat, v_hat with ka = k2**(alpv/2) per element   -> k_uv
//   nlt.f90:41-43   3 x cufftExecZ2D in place        (fft_inv.f90:12)
//   nlt.f90:46      produ                            -> k_produ
//   nlt.f90:50-51   2 x cufftExecD2Z in place + /NY/NX per array (fft_dir.f90:12-21) -> k_scale
//   nlt.f90:54-61   divergence                       -> k_div
//   nlt.f90:63      trunc: ellipse test with 2 divisions per element + mean=0 -> k_trunc, k_mean
//   rkstep.f90      copy, stage kernels, (1,1)=0 kernels; emk read from a table
//   forcing.f90     one device thread, serial LCG + sin/cos -> k_forcing_serial
// Everything runs on one stream (the reference's cuFFT streams are blocking streams ordered
// against the OpenACC default queue).
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "../include/gturbo.h"

struct re_handle {
  gt_params p;
  int N, NH, rko, nf;
  double dt2, dt3, dt6, sdt, fkxsmax, fkysmax, rtrunc2;
  cufftHandle pinv, pdir;
  cudaStream_t stream;
  double *fkx, *fky, *fkxs, *fkys, *emk;
  int *jc, *ikxf, *ikyf;
  int32_t* seed;
};

namespace {

constexpr int TB = 256;
int grid(size_t n) { return (int)((n + TB - 1) / TB > 4096 ? 4096 : (n + TB - 1) / TB); }

__global__ void k_uv(const double* z, double* u, double* v, const double* fkx, const double* fky,
                     const double* fkxs, const double* fkys, int N, int NH, double alpv) {
  const size_t tot = (size_t)N * NH;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < tot; o += (size_t)gridDim.x * blockDim.x) {
    if (o == 0) continue;
    const int j = (int)(o / NH), i = (int)(o % NH);
    const double k2 = fkxs[i] + fkys[j];
    const double ka = pow(k2, alpv / 2.0);
    const double kx = fkx[i] / ka, ky = fky[j] / ka;
    u[2 * o] = -ky * z[2 * o + 1];
    u[2 * o + 1] = ky * z[2 * o];
    v[2 * o] = kx * z[2 * o + 1];
    v[2 * o + 1] = -kx * z[2 * o];
  }
}

__global__ void k_produ(const double* z, double* u, double* v, int N) {
  const size_t ns = (size_t)(N + 2), tot = ns * N;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < tot; o += (size_t)gridDim.x * blockDim.x) {
    if ((int)(o % ns) < N) {
      u[o] = z[o] * u[o];
      v[o] = z[o] * v[o];
    } else {
      u[o] = 0.0;
      v[o] = 0.0;
    }
  }
}

__global__ void k_scale(double* z, int N) {
  const size_t tot = (size_t)(N + 2) * N;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < tot; o += (size_t)gridDim.x * blockDim.x)
    z[o] = z[o] / N / N;
}

__global__ void k_div(double* z, const double* u, const double* v, const double* fkx, const double* fky,
                      int N, int NH) {
  const size_t tot = (size_t)N * NH;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < tot; o += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(o / NH), i = (int)(o % NH);
    z[2 * o] = fkx[i] * u[2 * o + 1] + fky[j] * v[2 * o + 1];
    z[2 * o + 1] = -fkx[i] * u[2 * o] - fky[j] * v[2 * o];
  }
}

__global__ void k_trunc(double* z, const double* fkxs, const double* fkys, double fkxsmax,
                        double fkysmax, double rtrunc2, int N, int NH) {
  const size_t tot = (size_t)N * NH;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < tot; o += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(o / NH), i = (int)(o % NH);
    const double k1 = fkys[j] / fkysmax;
    const double k2 = k1 + fkxs[i] / fkxsmax;
    if (k2 > rtrunc2) {
      z[2 * o] = 0.0;
      z[2 * o + 1] = 0.0;
    }
  }
}

__global__ void k_zero_mean(double* z) {
  z[0] = 0.0;
  z[1] = 0.0;
}

// RK2 stage kernels (rkstep.f90:31-37, 61-67)
__global__ void k_rk2a(const double* z, double* znl, const double* emk, double dt2, size_t nc) {
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < nc; o += (size_t)gridDim.x * blockDim.x) {
    znl[2 * o] = emk[o] * (z[2 * o] + dt2 * znl[2 * o]);
    znl[2 * o + 1] = emk[o] * (z[2 * o + 1] + dt2 * znl[2 * o + 1]);
  }
}
__global__ void k_rk2b(double* z, const double* znl, const double* emk, double dt, size_t nc) {
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < nc; o += (size_t)gridDim.x * blockDim.x) {
    z[2 * o] = emk[o] * (emk[o] * z[2 * o] + dt * znl[2 * o]);
    z[2 * o + 1] = emk[o] * (emk[o] * z[2 * o + 1] + dt * znl[2 * o + 1]);
  }
}
// RK4 array statements (rkstep.f90:95-124), one kernel each
__global__ void k_rk4(int which, double* z, double* znl, double* znew, const double* emk, double dt,
                      double dt2, double dt3, double dt6, size_t nc) {
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < nc; o += (size_t)gridDim.x * blockDim.x) {
    const double e = emk[o];
    for (int c = 0; c < 2; ++c) {
      const size_t q = 2 * o + c;
      switch (which) {
        case 0: znew[q] = e * e * (z[q] + dt6 * znl[q]); break;
        case 1: znl[q] = e * (z[q] + dt2 * znl[q]); break;
        case 2: znew[q] = znew[q] + dt3 * e * znl[q]; break;
        case 3: znl[q] = e * z[q] + dt2 * znl[q]; break;
        case 4: znl[q] = e * (e * z[q] + dt * znl[q]); break;
        case 5: z[q] = znew[q] + dt6 * znl[q]; break;
      }
    }
  }
}

// forcing.f90:16-33: a single device thread walks the forced modes with the serial LCG.
__global__ void k_forcing_serial(double* z, int32_t* seed, const int* ikxf, const int* ikyf,
                                 const int* jc, int nf, int NH, double sf) {
  const double pi2 = 2.0 * 3.14159265358979;
  uint32_t x = (uint32_t)(*seed);
  for (int k = 0; k < nf; ++k) {
    x = (69069u * x + 1u) & 0x7FFFFFFFu;
    const float r = (float)((double)x / 2147483647.0);
    const double te = pi2 * (double)r;
    const double cc = cos(te), cs = sin(te);
    const int i = ikxf[k], j = ikyf[k];
    const size_t o = 2 * ((size_t)j * NH + i);
    z[o] = z[o] + sf * cc;
    z[o + 1] = z[o + 1] + sf * cs;
    if (i == 0 || i == NH - 1) {
      const size_t oc = 2 * ((size_t)jc[j] * NH + i);
      z[oc] = z[oc] + sf * cc;
      z[oc + 1] = z[oc + 1] - sf * cs;
    }
  }
  *seed = (int32_t)x;
}

int nlt(re_handle* h, double* z, double* u, double* v) {
  const int N = h->N, NH = h->NH;
  const size_t bytes = sizeof(double) * (size_t)(N + 2) * N;
  const size_t nc = (size_t)N * NH;
  cudaStream_t s = h->stream;
  cudaMemsetAsync(u, 0, bytes, s);
  cudaMemsetAsync(v, 0, bytes, s);
  k_uv<<<grid(nc), TB, 0, s>>>(z, u, v, h->fkx, h->fky, h->fkxs, h->fkys, N, NH, h->p.alpv);
  if (cufftExecZ2D(h->pinv, (cufftDoubleComplex*)z, z)) return 1;
  if (cufftExecZ2D(h->pinv, (cufftDoubleComplex*)v, v)) return 1;
  if (cufftExecZ2D(h->pinv, (cufftDoubleComplex*)u, u)) return 1;
  k_produ<<<grid((size_t)(N + 2) * N), TB, 0, s>>>(z, u, v, N);
  if (cufftExecD2Z(h->pdir, u, (cufftDoubleComplex*)u)) return 1;
  k_scale<<<grid((size_t)(N + 2) * N), TB, 0, s>>>(u, N);
  if (cufftExecD2Z(h->pdir, v, (cufftDoubleComplex*)v)) return 1;
  k_scale<<<grid((size_t)(N + 2) * N), TB, 0, s>>>(v, N);
  k_div<<<grid(nc), TB, 0, s>>>(z, u, v, h->fkx, h->fky, N, NH);
  if (h->p.truncate == 1) {
    k_trunc<<<grid(nc), TB, 0, s>>>(z, h->fkxs, h->fkys, h->fkxsmax, h->fkysmax, h->rtrunc2, N, NH);
    k_zero_mean<<<1, 1, 0, s>>>(z);
  }
  return cudaGetLastError() != cudaSuccess;
}

}  // namespace

extern "C" {

int re_create(const gt_params* p, re_handle** out) {
  re_handle* h = new (std::nothrow) re_handle();
  if (!h) return GT_ERR_NOMEM;
  std::memset(h, 0, sizeof(*h));
  h->p = *p;
  const int N = h->N = p->n, NH = h->NH = N / 2 + 1;
  h->rko = p->rko == 4 ? 4 : 2;
  h->dt2 = p->dt / 2.0;
  h->dt3 = p->dt / 3.0;
  h->dt6 = p->dt / 6.0;
  h->sdt = std::sqrt(p->dt);
  std::vector<double> fkx(NH), fky(N), fkxs(NH), fkys(N), emk((size_t)N * NH);
  std::vector<int> jc(N), ikxf, ikyf;
  const double dkx = 2.0 * 3.14159265358979323846 / p->xlx, dky = 2.0 * 3.14159265358979323846 / p->xly;
  for (int i = 0; i < NH; ++i) { fkx[i] = i * dkx; fkxs[i] = fkx[i] * fkx[i]; }
  for (int j = 0; j < N; ++j) {
    fky[j] = (j <= N / 2 ? j : j - N) * dky;
    fkys[j] = fky[j] * fky[j];
    jc[j] = j == 0 ? 0 : N - j;
  }
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < NH; ++i) {
      if (!i && !j) { emk[0] = 0.0; continue; }
      const double fk2 = fkxs[i] + fkys[j];
      emk[(size_t)j * NH + i] = std::exp(-0.5 * p->dt * (p->nu * std::pow(fk2, p->alpnu) + p->mu * std::pow(fk2, p->alpmu)));
    }
  h->fkxsmax = fkxs[N / 2];
  h->fkysmax = fkys[N / 2];
  h->rtrunc2 = p->rtrunc * p->rtrunc;
  for (int pass = 0; pass < 3; ++pass) {
    const int ilo = pass == 0 ? 0 : pass == 1 ? 1 : N / 2, ihi = pass == 0 ? 0 : pass == 1 ? N / 2 - 1 : N / 2;
    for (int i = ilo; i <= ihi; ++i)
      for (int j = pass == 0 ? 1 : 0; j <= (pass == 1 ? N - 1 : N / 2); ++j) {
        const double k2 = fkxs[i] + fkys[j], k2n = fkxs[i] / h->fkxsmax + fkys[j] / h->fkysmax;
        if (k2n <= h->rtrunc2 && k2 <= p->k2f * p->k2f && k2 > p->k1f * p->k1f) {
          ikxf.push_back(i);
          ikyf.push_back(j);
        }
      }
  }
  h->nf = (int)ikxf.size();
  if (h->nf > GT_NFORC) { delete h; return GT_ERR_NFORC; }
  auto up = [](void** d, const void* s, size_t b) {
    if (cudaMalloc(d, b ? b : 8)) return 1;
    return s && b ? (int)cudaMemcpy(*d, s, b, cudaMemcpyHostToDevice) : 0;
  };
  int rc = 0;
  rc |= up((void**)&h->fkx, fkx.data(), 8 * NH);
  rc |= up((void**)&h->fky, fky.data(), 8 * N);
  rc |= up((void**)&h->fkxs, fkxs.data(), 8 * NH);
  rc |= up((void**)&h->fkys, fkys.data(), 8 * N);
  rc |= up((void**)&h->emk, emk.data(), 8 * emk.size());
  rc |= up((void**)&h->jc, jc.data(), 4 * N);
  rc |= up((void**)&h->ikxf, ikxf.data(), 4 * ikxf.size());
  rc |= up((void**)&h->ikyf, ikyf.data(), 4 * ikyf.size());
  rc |= up((void**)&h->seed, nullptr, 4);
  rc |= cufftPlan2d(&h->pinv, N, N, CUFFT_Z2D) != CUFFT_SUCCESS;
  rc |= cufftPlan2d(&h->pdir, N, N, CUFFT_D2Z) != CUFFT_SUCCESS;
  if (rc) { delete h; return GT_ERR_CUDA; }
  *out = h;
  return GT_OK;
}

int re_set_stream(re_handle* h, void* stream) {
  h->stream = (cudaStream_t)stream;
  if (cufftSetStream(h->pinv, h->stream) || cufftSetStream(h->pdir, h->stream)) return GT_ERR_CUDA;
  return GT_OK;
}

int re_destroy(re_handle* h) {
  if (!h) return GT_OK;
  cudaDeviceSynchronize();
  cufftDestroy(h->pinv);
  cufftDestroy(h->pdir);
  void* ptrs[] = {h->fkx, h->fky, h->fkxs, h->fkys, h->emk, h->jc, h->ikxf, h->ikyf, h->seed};
  for (void* q : ptrs) cudaFree(q);
  delete h;
  return GT_OK;
}

int re_nlt(re_handle* h, double* z, double* u, double* v) { return nlt(h, z, u, v) ? GT_ERR_CUDA : GT_OK; }

// step / step4 (rkstep.f90:2-131) with the split=0 integrating factor.
int re_step(re_handle* h, double* z, double* znl, double* znew, double* u, double* v) {
  const int N = h->N;
  const size_t nc = (size_t)N * h->NH, bytes = sizeof(double) * (size_t)(N + 2) * N;
  cudaStream_t s = h->stream;
  const double dt = h->p.dt;
  cudaMemcpyAsync(znl, z, bytes, cudaMemcpyDeviceToDevice, s);
  if (nlt(h, znl, u, v)) return GT_ERR_CUDA;
  if (h->rko == 4) {
    k_rk4<<<grid(nc), TB, 0, s>>>(0, z, znl, znew, h->emk, dt, h->dt2, h->dt3, h->dt6, nc);
    k_rk4<<<grid(nc), TB, 0, s>>>(1, z, znl, znew, h->emk, dt, h->dt2, h->dt3, h->dt6, nc);
    if (nlt(h, znl, u, v)) return GT_ERR_CUDA;
    k_rk4<<<grid(nc), TB, 0, s>>>(2, z, znl, znew, h->emk, dt, h->dt2, h->dt3, h->dt6, nc);
    k_rk4<<<grid(nc), TB, 0, s>>>(3, z, znl, znew, h->emk, dt, h->dt2, h->dt3, h->dt6, nc);
    if (nlt(h, znl, u, v)) return GT_ERR_CUDA;
    k_rk4<<<grid(nc), TB, 0, s>>>(2, z, znl, znew, h->emk, dt, h->dt2, h->dt3, h->dt6, nc);
    k_rk4<<<grid(nc), TB, 0, s>>>(4, z, znl, znew, h->emk, dt, h->dt2, h->dt3, h->dt6, nc);
    if (nlt(h, znl, u, v)) return GT_ERR_CUDA;
    k_rk4<<<grid(nc), TB, 0, s>>>(5, z, znl, znew, h->emk, dt, h->dt2, h->dt3, h->dt6, nc);
    k_zero_mean<<<1, 1, 0, s>>>(z);
  } else {
    k_rk2a<<<grid(nc), TB, 0, s>>>(z, znl, h->emk, h->dt2, nc);
    k_zero_mean<<<1, 1, 0, s>>>(znl);
    if (nlt(h, znl, u, v)) return GT_ERR_CUDA;
    k_rk2b<<<grid(nc), TB, 0, s>>>(z, znl, h->emk, dt, nc);
    k_zero_mean<<<1, 1, 0, s>>>(z);
  }
  return cudaGetLastError() == cudaSuccess ? GT_OK : GT_ERR_CUDA;
}

// forcing with the LCG state kept on the device, as the reference's `!$acc copyin(seed)`.
int re_set_seed(re_handle* h, int32_t seed) {
  return cudaMemcpyAsync(h->seed, &seed, 4, cudaMemcpyHostToDevice, h->stream) == cudaSuccess ? GT_OK : GT_ERR_CUDA;
}
int re_get_seed(re_handle* h, int32_t* seed) {
  if (cudaMemcpyAsync(seed, h->seed, 4, cudaMemcpyDeviceToHost, h->stream)) return GT_ERR_CUDA;
  return cudaStreamSynchronize(h->stream) == cudaSuccess ? GT_OK : GT_ERR_CUDA;
}
int re_forcing(re_handle* h, double* z) {
  if (h->nf == 0) return GT_OK;
  k_forcing_serial<<<1, 1, 0, h->stream>>>(z, h->seed, h->ikxf, h->ikyf, h->jc, h->nf, h->NH,
                                            h->sdt * h->p.famp);
  return cudaGetLastError() == cudaSuccess ? GT_OK : GT_ERR_CUDA;
}

}  // extern "C"
