// Axion power spectrum pieces of specific_post_timestep
// (AxionStringsLevel.cpp:1583-1640): the masked a_dot buffer
// (MaskedFieldBuffer.hpp:15-35) and the shell binning of its R2C transform
// (SpectrumKernel.hpp:53-153). The FFT between them is a plain library R2C
// (cuFFT), unnormalised forward, the convention the reference's binning uses.
//
// Binning is deterministic: each warp keeps its own shell histogram in shared
// memory; lanes holding the same shell are grouped with __match_any_sync and
// their values summed in lane order by the group leader; warp histograms are
// summed in warp order into one partial per block, and the partials in block
// order by a one-block finalise.
#include <algorithm>
#include <cmath>

#include "axs_internal.cuh"

namespace axs {

int level_geom(int32_t dtype, int nx, int ny, int nz, LevelGeom &g);

constexpr int kSpecThreads = 256, kSpecWarps = kSpecThreads / 32;

static int spec_grid()
{
    const int sms = device_sm_count() > 0 ? device_sm_count() : 148;
    return sms * 2;
}

static int n_shells_for(int nx, int ny, int nz) { return std::max(nx, std::max(ny, nz)) / 2 + 1; }

// masked_a_dot (Masking.hpp:96-118) with round-to-nearest double operations,
// so the buffer equals the CPU evaluation bit for bit.
__device__ __forceinline__ double masked_a_dot_rn(int scheme, double thr, double p1, double p2, double q1, double q2,
                                                  double R)
{
    const double raw = __dsub_rn(__dmul_rn(p1, q2), __dmul_rn(q1, p2));
    if (scheme == AXS_MASK_A) return raw;
    const double psi_sq = __dadd_rn(__dmul_rn(p1, p1), __dmul_rn(p2, p2));
    if (scheme == AXS_MASK_B && !(__ddiv_rn(__dsqrt_rn(psi_sq), R) >= thr)) return 0.0;
    return __ddiv_rn(raw, psi_sq);
}

template <typename T>
__global__ void __launch_bounds__(kSpecThreads) masked_a_dot_kernel(const T *__restrict__ st, LevelGeom g, int nx,
                                                                    int ny, int nz, int scheme, double thr, double R,
                                                                    T *__restrict__ buf, double *__restrict__ part)
{
    const int64_t n = (int64_t)nx * ny * nz;
    double acc = 0.0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % nx), j = (int)((c / nx) % ny), k = (int)(c / ((int64_t)nx * ny));
        const int64_t o = (i + g.ox) + (int64_t)(j + g.oy) * g.js + (int64_t)k * g.ks;
        const T v = (T)masked_a_dot_rn(scheme, thr, st[o], st[g.cs + o], st[2 * g.cs + o], st[3 * g.cs + o], R);
        buf[c] = v;
        acc += (double)v * (double)v;
    }
    __shared__ double red[kSpecThreads];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kSpecThreads / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void sum_partials_fixed(const double *__restrict__ part, int n, double *__restrict__ out)
{
    __shared__ double red[kSpecThreads];
    double x = 0.0;
    for (int i = threadIdx.x; i < n; i += kSpecThreads) x += part[i];
    red[threadIdx.x] = x;
    __syncthreads();
    for (int s = kSpecThreads / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// Per-block shell partials: part[b * (2 S + 2) + s] = shell sums, [S + s] = counts,
// [2 S] = full-cube energy, [2 S + 1] = inscribed-sphere energy.
template <typename T>
__global__ void __launch_bounds__(kSpecThreads) spectrum_bin_kernel(const T *__restrict__ spec, int nx, int ny, int nz,
                                                                    int S, double *__restrict__ part)
{
    extern __shared__ double hist[];  // [kSpecWarps][2 S]
    __shared__ int lane_shell[kSpecWarps][32];
    __shared__ double lane_val[kSpecWarps][32];
    __shared__ double lane_cnt[kSpecWarps][32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int s = tid; s < kSpecWarps * 2 * S; s += kSpecThreads) hist[s] = 0.0;
    __syncthreads();
    const int nxh = nx / 2 + 1;
    const int64_t nmodes = (int64_t)nxh * ny * nz;
    const int n_max = max(nx, max(ny, nz));
    const double half = 0.5 * n_max, four_pi = 4.0 * 3.14159265358979323846;
    double full = 0.0, insc = 0.0;
    double *h = hist + (size_t)warp * 2 * S;
    const int64_t stride = (int64_t)gridDim.x * kSpecThreads;
    for (int64_t base = ((int64_t)blockIdx.x * kSpecWarps + warp) * 32; base < nmodes; base += stride) {
        const int64_t m = base + lane;
        int shell = -1;
        double val = 0.0, cw = 0.0;
        if (m < nmodes) {
            const int i = (int)(m % nxh), j = (int)((m / nxh) % ny), k = (int)(m / ((int64_t)nxh * ny));
            const int kx = i, ky = j <= ny / 2 ? j : j - ny, kz = k <= nz / 2 ? k : k - nz;
            const double p_sq = (double)(kx * kx + ky * ky + kz * kz);
            const double p = sqrt(p_sq);
            const double re = spec[2 * m], im = spec[2 * m + 1];
            const double mag = re * re + im * im;
            const double w = (kx == 0 || kx == nx / 2) ? 1.0 : 2.0;
            full += w * mag;
            if (p < half) {
                insc += w * mag;
                const int sh = (int)floor(p + 0.5);
                if (sh < S) {
                    shell = sh;
                    val = w * four_pi * p_sq * mag;
                    cw = w;
                }
            }
        }
        lane_shell[warp][lane] = shell;
        lane_val[warp][lane] = val;
        lane_cnt[warp][lane] = cw;
        __syncwarp();
        const unsigned grp = __match_any_sync(0xffffffffu, shell);
        if (shell >= 0 && lane == __ffs(grp) - 1) {
            double sv = 0.0, sc = 0.0;
            for (unsigned b = grp; b; b &= b - 1) {
                const int l = __ffs(b) - 1;
                sv += lane_val[warp][l];
                sc += lane_cnt[warp][l];
            }
            h[shell] += sv;
            h[S + shell] += sc;
        }
        __syncwarp();
    }
    __syncthreads();
    double *out = part + (size_t)blockIdx.x * (2 * S + 2);
    for (int s = tid; s < 2 * S; s += kSpecThreads) {
        double x = 0.0;
        for (int w = 0; w < kSpecWarps; ++w) x += hist[(size_t)w * 2 * S + s];
        out[s] = x;
    }
    __shared__ double red[2][kSpecThreads];
    red[0][tid] = full;
    red[1][tid] = insc;
    __syncthreads();
    for (int s = kSpecThreads / 2; s > 0; s >>= 1) {
        if (tid < s) {
            red[0][tid] += red[0][tid + s];
            red[1][tid] += red[1][tid + s];
        }
        __syncthreads();
    }
    if (tid == 0) {
        out[2 * S] = red[0][0];
        out[2 * S + 1] = red[1][0];
    }
}

__global__ void spectrum_finalize_kernel(const double *__restrict__ part, int nblocks, int S,
                                         double *__restrict__ shell_sum, int64_t *__restrict__ shell_count,
                                         double *__restrict__ totals)
{
    for (int s = threadIdx.x; s < 2 * S + 2; s += blockDim.x) {
        double x = 0.0;
        for (int b = 0; b < nblocks; ++b) x += part[(size_t)b * (2 * S + 2) + s];
        if (s < S)
            shell_sum[s] = x;
        else if (s < 2 * S)
            shell_count[s - S] = (int64_t)llrint(x);
        else
            totals[s - 2 * S] = x;
    }
}

}  // namespace axs

using namespace axs;

extern "C" {

int axs_spectrum_scratch_bytes(int32_t nx, int32_t ny, int32_t nz, int64_t *bytes)
{
    AXS_REQUIRE(bytes != nullptr && nx > 0 && ny > 0 && nz > 0, AXS_ERR_INVALID_ARGUMENT, "bad arguments");
    const int S = n_shells_for(nx, ny, nz);
    *bytes = (int64_t)spec_grid() * (2 * S + 2) * (int64_t)sizeof(double);
    return AXS_OK;
}

int axs_level_masked_a_dot(const axs_level *lv, int32_t masking_scheme, double masking_threshold, double R,
                           void *buf_dev, double *sum_sq_dev, void *scratch, int64_t scratch_bytes, void *stream)
{
    AXS_REQUIRE(lv != nullptr && lv->state != nullptr && buf_dev != nullptr && sum_sq_dev != nullptr,
                AXS_ERR_INVALID_ARGUMENT, "null argument");
    AXS_REQUIRE(masking_scheme >= AXS_MASK_NONE && masking_scheme <= AXS_MASK_B, AXS_ERR_INVALID_ARGUMENT,
                "bad masking scheme %d", masking_scheme);
    AXS_REQUIRE(R > 0.0, AXS_ERR_INVALID_ARGUMENT, "R must be positive");
    LevelGeom g;
    int rc = level_geom(lv->dtype, lv->nx, lv->ny, lv->nz, g);
    if (rc) return rc;
    const int grid = spec_grid();
    AXS_REQUIRE(scratch != nullptr && scratch_bytes >= (int64_t)grid * 8, AXS_ERR_WORKSPACE,
                "masked buffer scratch needs %d bytes", grid * 8);
    cudaStream_t st = (cudaStream_t)stream;
    double *part = static_cast<double *>(scratch);
    if (lv->dtype == AXS_F32)  // fill_masked_a_dot_buffer takes R as amrex::Real
        masked_a_dot_kernel<float><<<grid, kSpecThreads, 0, st>>>(static_cast<const float *>(lv->state), g, lv->nx,
                                                                  lv->ny, lv->nz, masking_scheme, masking_threshold,
                                                                  (double)(float)R, static_cast<float *>(buf_dev), part);
    else
        masked_a_dot_kernel<double><<<grid, kSpecThreads, 0, st>>>(static_cast<const double *>(lv->state), g, lv->nx,
                                                                   lv->ny, lv->nz, masking_scheme, masking_threshold, R,
                                                                   static_cast<double *>(buf_dev), part);
    if ((rc = launch_status("masked a_dot buffer"))) return rc;
    sum_partials_fixed<<<1, kSpecThreads, 0, st>>>(part, grid, sum_sq_dev);
    return launch_status("masked a_dot sum");
}

int axs_spectrum_bin(const void *spec_dev, int32_t dtype, int32_t nx, int32_t ny, int32_t nz, double *shell_sum_dev,
                     int64_t *shell_count_dev, double *totals_dev, void *scratch, int64_t scratch_bytes,
                     void *stream)
{
    AXS_REQUIRE(spec_dev && shell_sum_dev && shell_count_dev && totals_dev, AXS_ERR_INVALID_ARGUMENT,
                "null argument");
    AXS_REQUIRE(dtype == AXS_F32 || dtype == AXS_F64, AXS_ERR_INVALID_ARGUMENT, "bad dtype %d", dtype);
    AXS_REQUIRE(nx > 0 && ny > 0 && nz > 0, AXS_ERR_INVALID_ARGUMENT, "empty domain");
    int64_t need = 0;
    axs_spectrum_scratch_bytes(nx, ny, nz, &need);
    AXS_REQUIRE(scratch != nullptr && scratch_bytes >= need, AXS_ERR_WORKSPACE,
                "spectrum scratch too small (%lld < %lld)", (long long)scratch_bytes, (long long)need);
    const int S = n_shells_for(nx, ny, nz);
    const size_t smem = (size_t)kSpecWarps * 2 * S * sizeof(double);
    AXS_REQUIRE(smem <= 200 * 1024, AXS_ERR_UNSUPPORTED, "too many shells (%d) for the shared histograms", S);
    cudaStream_t st = (cudaStream_t)stream;
    const int grid = spec_grid();
    double *part = static_cast<double *>(scratch);
    int rc;
    if (dtype == AXS_F32) {
        AXS_CUDA_CHECK(cudaFuncSetAttribute(spectrum_bin_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem));
        spectrum_bin_kernel<float><<<grid, kSpecThreads, smem, st>>>(static_cast<const float *>(spec_dev), nx, ny, nz,
                                                                     S, part);
    } else {
        AXS_CUDA_CHECK(cudaFuncSetAttribute(spectrum_bin_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem));
        spectrum_bin_kernel<double><<<grid, kSpecThreads, smem, st>>>(static_cast<const double *>(spec_dev), nx, ny,
                                                                      nz, S, part);
    }
    if ((rc = launch_status("spectrum binning"))) return rc;
    spectrum_finalize_kernel<<<1, kSpecThreads, 0, st>>>(part, grid, S, shell_sum_dev, shell_count_dev, totals_dev);
    return launch_status("spectrum finalize");
}

}  // extern "C"
