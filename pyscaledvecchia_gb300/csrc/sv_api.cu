// Library-wide helpers of the C ABI: status strings, error recording, device
// properties, and the elementwise Matern / Bessel entry points.
#include <stdio.h>

#include "sv_common.cuh"
#include "sv_matern.cuh"

static thread_local int g_last_cuda_error = 0;

int sv_record_cuda_error(cudaError_t e) {
  g_last_cuda_error = (int)e;
  return SV_ECUDA;
}

int sv_num_sms() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (cached[dev] <= 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = v > 0 ? v : 1;
  }
  return cached[dev];
}

extern "C" const char* sv_status_string(int s) {
  switch (s) {
    case SV_OK: return "ok";
    case SV_EINVAL: return "invalid argument or unsupported size";
    case SV_ECHOL: return "block Cholesky failed even with jitter";
    case SV_ETIMEOUT: return "a bounded device wait ran out";
    case SV_ECUDA: return "CUDA runtime error";
    case SV_ENOSPC: return "workspace too small";
    default: return "unknown status";
  }
}

extern "C" int sv_abi_version(void) { return SV_ABI_VERSION; }

extern "C" int sv_last_cuda_error(void) { return g_last_cuda_error; }

namespace sv {

__global__ void k_matern_eval(const double* r, int64_t n, double nu, int which, int general,
                              double log_coef, int code, double* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double ri = r[i];
    double M, g;
    if (general) {
      if (which == 0)
        M = matern_general_M(ri, nu, log_coef), g = 0.0;
      else
        matern_general_Mg(ri, nu, log_coef, M, g);
    } else if (which == 1 && code == 0) {
      // _covariance.py:63-66 (nu = 0.5): g = -exp(-r)/r for r > 0, else 0
      matern_closed(code, ri, M, g);
    } else {
      matern_closed(code, ri, M, g);
    }
    out[i] = which == 0 ? M : g;
  }
}

// the split kernels' float32 Matern at r rounded to float32: which = 2 the
// deficit D = 1 - M, which = 3 g, which = 4 dM/dnu of an estimated nu (the
// central difference at nu +- 1e-3); a closed form (general = 0) or the
// float32 tables of a general nu, which every CTA builds in its shared
// memory as the likelihood's table kernel builds them in global memory
__global__ void k_matern_eval32(const double* r, int64_t n, double nu, int which, int general,
                                int code, double* out) {
  __shared__ double fv[3][kFtabIntervals * kFtabN];
  __shared__ __align__(16) float tab[kFtabMaxFloats];
  __shared__ __align__(16) float dtab[kDtabMaxFloats];
  MaternF32 mf;
  mf.code = general ? 3 : code;
  mf.elo = general ? mtab_elo(nu) : 0;
  mf.esw = ftab_switch(nu);
  mf.s2n = (float)sqrt(2.0 * nu);
  mf.tab = (const float4*)tab;
  mf.dtab = which == 4 ? (const float4*)dtab : nullptr;
  mf.nuf = (float)nu;
  if (general) {
    const int nint = ftab_intervals(mf.elo);
    for (int t = threadIdx.x; t < nint * kFtabN; t += blockDim.x) {
      ftab_node(nu, mf.elo, mf.esw, t / kFtabN, t % kFtabN, fv[0][t], fv[1][t]);
      if (which == 4) fv[2][t] = ftab_dnu_node(nu, 1e-3, mf.elo, mf.esw, t / kFtabN, t % kFtabN);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nint * 2 * kFtabN; t += blockDim.x) {
      const int iv = t / (2 * kFtabN), w = (t / kFtabN) & 1, j = t % kFtabN;
      tab[t] = ftab_coef(fv[w] + iv * kFtabN, j);
    }
    if (which == 4)
      for (int t = threadIdx.x; t < nint * kFtabN; t += blockDim.x)
        dtab[t] = ftab_coef(fv[2] + (t / kFtabN) * kFtabN, t % kFtabN);
    __syncthreads();
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float rf = (float)r[i];
    const float v = which == 2 ? matern_deficit_f32(mf, rf)
                    : which == 3 ? matern_g_f32(mf, rf)
                                 : matern_dnu_f32(mf, rf);
    out[i] = (double)v;
  }
}

// the float64 Matern table of nu (as the likelihood builds it): CTA
// (interval) of kMtabN threads
__global__ void k_matern_table1(double nu, double* tab) {
  __shared__ double fm[kMtabN], fg[kMtabN];
  mtab_build_interval(nu, blockIdx.x, fm, fg, tab);
}

// its float32 part (the split prediction blocks): CTA (interval) of kFtabN
// threads, as the likelihood's float32 tables
__global__ void k_matern_ftab1(double nu, float* ft) {
  __shared__ double ff[kFtabN], fq[kFtabN];
  const int iv = blockIdx.x, j = threadIdx.x;
  ftab_node(nu, mtab_elo(nu), ftab_switch(nu), iv, j, ff[j], fq[j]);
  __syncthreads();
  ft[(size_t)iv * 2 * kFtabN + j] = ftab_coef(ff, j);
  ft[(size_t)iv * 2 * kFtabN + kFtabN + j] = ftab_coef(fq, j);
}

__global__ void k_bessel_k(const double* x, int64_t n, double nu, double* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = bessel_k(nu, x[i]);
}

// 8 independent float64 FMA chains per thread (peak-rate measurement)
__global__ void k_fp64_probe(double* out, int iters) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5,
         a6 = a0 + 6, a7 = a0 + 7;
  const double s = 0.999999;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, s, 1e-9);
    a1 = fma(a1, s, 1e-9);
    a2 = fma(a2, s, 1e-9);
    a3 = fma(a3, s, 1e-9);
    a4 = fma(a4, s, 1e-9);
    a5 = fma(a5, s, 1e-9);
    a6 = fma(a6, s, 1e-9);
    a7 = fma(a7, s, 1e-9);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

// 8 independent float32 FMA chains per thread (peak-rate measurement of the
// FP32 pipe, which carries the split kernel's double-float arithmetic)
__global__ void k_fp32_probe(float* out, int iters) {
  float a0 = threadIdx.x * 1e-3f, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5,
        a6 = a0 + 6, a7 = a0 + 7;
  const float s = 0.999999f;
  for (int i = 0; i < iters; ++i) {
    a0 = __fmaf_rn(a0, s, 1e-9f);
    a1 = __fmaf_rn(a1, s, 1e-9f);
    a2 = __fmaf_rn(a2, s, 1e-9f);
    a3 = __fmaf_rn(a3, s, 1e-9f);
    a4 = __fmaf_rn(a4, s, 1e-9f);
    a5 = __fmaf_rn(a5, s, 1e-9f);
    a6 = __fmaf_rn(a6, s, 1e-9f);
    a7 = __fmaf_rn(a7, s, 1e-9f);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

}  // namespace sv

extern "C" int sv_device_reads_host_memory(int32_t* out) {
  if (!out) return SV_EINVAL;
  int dev = 0, pageable = 0, host_tables = 0;
  SV_CUDA_TRY(cudaGetDevice(&dev));
  SV_CUDA_TRY(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
  SV_CUDA_TRY(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
  *out = (pageable && host_tables) ? 1 : 0;
  return SV_OK;
}

extern "C" int64_t sv_fp64_probe_threads(void) { return 8LL * sv_num_sms() * 256; }

extern "C" int sv_fp32_fma_probe(float* out, int32_t iters, sv_stream_t stream) {
  if (!out || iters < 1) return SV_EINVAL;
  sv::k_fp32_probe<<<8 * sv_num_sms(), 256, 0, (cudaStream_t)stream>>>(out, iters);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

extern "C" int sv_fp64_fma_probe(double* out, int32_t iters, sv_stream_t stream) {
  if (!out || iters < 1) return SV_EINVAL;
  sv::k_fp64_probe<<<8 * sv_num_sms(), 256, 0, (cudaStream_t)stream>>>(out, iters);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

extern "C" int sv_matern_eval(const double* r, int64_t n, double nu, int32_t which,
                              int32_t general, double* out, sv_stream_t stream) {
  if (n < 0 || (n > 0 && (!r || !out)) || which < 0 || which > 4) return SV_EINVAL;
  if (!(nu > 0.0)) return SV_EINVAL;
  const int code = sv::matern_closed_code(nu);
  if (!general && code < 0) return SV_EINVAL;
  if (which >= 2 && general && !sv::ftab_ok(nu)) return SV_EINVAL;
  if (which == 4 && !(general && sv::ftab_est_ok(nu, 1e-3))) return SV_EINVAL;
  if (n == 0) return SV_OK;
  if (which >= 2) {
    int64_t grid = (n + 255) / 256;
    if (grid > 2LL * sv_num_sms()) grid = 2LL * sv_num_sms();
    sv::k_matern_eval32<<<(int)grid, 256, 0, (cudaStream_t)stream>>>(r, n, nu, which, general,
                                                                      code, out);
    SV_CUDA_TRY(cudaGetLastError());
    return SV_OK;
  }
  const double lc = general ? sv::matern_log_coef(nu) : 0.0;
  int64_t grid = (n + 255) / 256;
  if (grid > 16LL * sv_num_sms()) grid = 16LL * sv_num_sms();
  sv::k_matern_eval<<<(int)grid, 256, 0, (cudaStream_t)stream>>>(r, n, nu, which, general, lc, code,
                                                                  out);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

extern "C" int64_t sv_matern_table_doubles(void) { return sv::kMtabMaxDoubles + sv::kFtabMaxFloats / 2; }

extern "C" int sv_matern_table(double nu, double* table, int64_t table_doubles, sv_stream_t stream) {
  if (!table || !sv::mtab_ok(nu) || table_doubles < sv_matern_table_doubles()) return SV_EINVAL;
  if ((reinterpret_cast<uintptr_t>(table) & 15) != 0) return SV_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  sv::k_matern_table1<<<sv::mtab_intervals(sv::mtab_elo(nu)), sv::kMtabN, 0, st>>>(nu, table);
  SV_CUDA_TRY(cudaGetLastError());
  if (sv::ftab_ok(nu)) {
    sv::k_matern_ftab1<<<sv::ftab_intervals(sv::mtab_elo(nu)), sv::kFtabN, 0, st>>>(
        nu, reinterpret_cast<float*>(table + sv::kMtabMaxDoubles));
    SV_CUDA_TRY(cudaGetLastError());
  }
  return SV_OK;
}

extern "C" int sv_bessel_k(const double* x, int64_t n, double nu, double* out, sv_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !out)) || !(nu >= 0.0) && !(nu < 0.0)) return SV_EINVAL;
  if (n == 0) return SV_OK;
  int64_t grid = (n + 255) / 256;
  if (grid > 16LL * sv_num_sms()) grid = 16LL * sv_num_sms();
  sv::k_bessel_k<<<(int)grid, 256, 0, (cudaStream_t)stream>>>(x, n, nu, out);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}
