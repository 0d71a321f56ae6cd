// C-ABI plumbing: error reporting, host-side background/xi models, tensor-map
// creation, and the two small device entry points that need no tiling
// (winding known-answer batch, Fourier-IC spectral fill).
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>

#include "axs_internal.cuh"

namespace axs {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

static std::atomic<uint32_t> g_wait_polls{AXS_DEFAULT_WAIT_POLLS};

uint32_t device_wait_polls() { return g_wait_polls.load(std::memory_order_relaxed); }

int device_sm_count()
{
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return n;
}

int validate_fab(const axs_fab *f, const char *name, int min_comp, int min_ng)
{
    AXS_REQUIRE(f != nullptr, AXS_ERR_INVALID_ARGUMENT, "%s: null descriptor", name);
    AXS_REQUIRE(f->data != nullptr, AXS_ERR_INVALID_ARGUMENT, "%s: null data pointer", name);
    AXS_REQUIRE(f->dtype == AXS_F32 || f->dtype == AXS_F64, AXS_ERR_INVALID_ARGUMENT, "%s: bad dtype %d", name,
                f->dtype);
    AXS_REQUIRE(f->nx > 0 && f->ny > 0 && f->nz > 0, AXS_ERR_INVALID_ARGUMENT, "%s: empty box %dx%dx%d", name,
                f->nx, f->ny, f->nz);
    AXS_REQUIRE(f->ng >= min_ng, AXS_ERR_INVALID_ARGUMENT, "%s: needs >= %d ghost layers, has %d", name, min_ng,
                f->ng);
    AXS_REQUIRE(f->ncomp >= min_comp, AXS_ERR_INVALID_ARGUMENT, "%s: needs >= %d components, has %d", name,
                min_comp, f->ncomp);
    const int64_t rx = f->nx + 2LL * f->ng, ry = f->ny + 2LL * f->ng, rz = f->nz + 2LL * f->ng;
    AXS_REQUIRE(f->jstride >= rx && f->kstride >= f->jstride * ry && f->cstride >= f->kstride * rz,
                AXS_ERR_INVALID_ARGUMENT, "%s: strides (%lld,%lld,%lld) too small for the box", name,
                (long long)f->jstride, (long long)f->kstride, (long long)f->cstride);
    return AXS_OK;
}

// ------------------------------------------------------------ background model
// Background.hpp:55-107, FlatBackground.hpp:34-43, PreEvolutionBackground.hpp:93-113.
static double bg_c(const axs_background &b, double tau)
{
    return (b.has_switch && tau >= b.tau_switch) ? b.c1 : b.c0;
}

static double bg_R(const axs_background &b, double tau)
{
    if (b.kind == AXS_BG_FLAT) return 1.0;
    if (b.kind == AXS_BG_PRE_EVOLUTION) return std::exp(tau);
    const double b_inv = b.a_inv - 1.0;
    return (1.0 / b_inv) * std::pow(tau, 1.0 / b_inv);
}

static double bg_R_prime(const axs_background &b, double tau)
{
    if (b.kind == AXS_BG_FLAT) return 0.0;
    if (b.kind == AXS_BG_PRE_EVOLUTION) return std::exp(tau);
    const double b_inv = b.a_inv - 1.0;
    return ((1.0 / b_inv) / b_inv) * std::pow(tau, 1.0 / b_inv - 1.0);
}

static double bg_lambda_unit(const axs_background &b, double tau)
{
    if (b.kind == AXS_BG_FLAT) return b.m_r * b.m_r;
    if (b.kind == AXS_BG_PRE_EVOLUTION) {
        const double r = std::exp(tau);
        return b.gamma_pre * b.gamma_pre / (r * r);
    }
    // lambda = lambda0 (R/R0)^(-2c), re-anchored at the switch (Background.hpp:75-86)
    const double R0 = 1.0 / (b.a_inv - 1.0);
    const double c_now = bg_c(b, tau);
    if (!b.has_switch || tau < b.tau_switch) return std::pow(bg_R(b, tau) / R0, -2.0 * c_now);
    const double R_s = bg_R(b, b.tau_switch);
    const double lambda_s = std::pow(R_s / R0, -2.0 * b.c0);
    return lambda_s * std::pow(bg_R(b, tau) / R_s, -2.0 * c_now);
}

static double bg_curvature(const axs_background &b, double tau)
{
    if (b.kind == AXS_BG_FLAT) return 0.0;
    if (b.kind == AXS_BG_PRE_EVOLUTION) return 1.0;
    const double b_inv = b.a_inv - 1.0;
    return (1.0 - b_inv) / (b_inv * b_inv * tau * tau);  // Background.hpp:67-70
}

void rhs_coeffs(const axs_background &b, double tau, axs_rhs_coeffs &c)
{
    double kappa = bg_curvature(b, tau);
    double lambda = b.lambda_scale * bg_lambda_unit(b, tau);
    if (b.kind == AXS_BG_EXPANDING && b.blend_dtau > 0.0) {
        // post-handoff smoothstep blend (AxionStringsLevel.cpp:893-906)
        const double t = (tau - b.blend_tau_start) / b.blend_dtau;
        if (t < 1.0) {
            const double tc = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
            const double s = tc * tc * (3.0 - 2.0 * tc);
            lambda = (1.0 - s) * b.blend_lambda_start + s * lambda;
            kappa = (1.0 - s) * b.blend_curv_start + s * kappa;
        }
    }
    const double R = bg_R(b, tau);
    c.kappa = kappa;
    c.lambda = lambda;
    c.R2 = (b.kind == AXS_BG_FLAT) ? 1.0 : R * R;
}

void background_values(const axs_background &b, double tau, axs_background_values &v)
{
    axs_rhs_coeffs c;
    rhs_coeffs(b, tau, c);
    v.R = bg_R(b, tau);
    v.R_prime = bg_R_prime(b, tau);
    v.kappa = c.kappa;
    v.lambda = c.lambda;
    v.H = v.R_prime / (v.R * v.R);
    v.R2 = c.R2;
    v.m_r = std::sqrt(c.lambda);
    v.R_prime_over_R = v.R_prime / v.R;
}

static int validate_background(const axs_background *bg)
{
    AXS_REQUIRE(bg != nullptr, AXS_ERR_INVALID_ARGUMENT, "null background");
    AXS_REQUIRE(bg->kind >= AXS_BG_EXPANDING && bg->kind <= AXS_BG_PRE_EVOLUTION, AXS_ERR_INVALID_ARGUMENT,
                "bad background kind %d", bg->kind);
    if (bg->kind == AXS_BG_EXPANDING)
        AXS_REQUIRE(bg->a_inv > 1.0, AXS_ERR_INVALID_ARGUMENT, "a_inv must exceed 1 (b_inv = a_inv - 1 > 0), got %g",
                    bg->a_inv);
    return AXS_OK;
}

// ------------------------------------------------------------ tensor maps
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

int make_tensor_map_4d(CUtensorMap *map, const void *base, int32_t dtype, uint64_t dim0, uint64_t dim1,
                       uint64_t dim2, uint64_t dim3, uint64_t stride1_bytes, uint64_t stride2_bytes,
                       uint64_t stride3_bytes, uint32_t box0, uint32_t box1, uint32_t box2, uint32_t box3)
{
    EncodeTiledFn fn = encode_fn();
    AXS_REQUIRE(fn != nullptr, AXS_ERR_CUDA, "cuTensorMapEncodeTiled unavailable from the driver");
    const cuuint64_t dims[4] = {dim0, dim1, dim2, dim3};
    const cuuint64_t strides[3] = {stride1_bytes, stride2_bytes, stride3_bytes};
    const cuuint32_t box[4] = {box0, box1, box2, box3};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = fn(map, dtype == AXS_F64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                          4, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    AXS_REQUIRE(r == CUDA_SUCCESS, AXS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return AXS_OK;
}

// ------------------------------------------------------------ device: winding KAT batch
// PlaquetteWinding.hpp:24-51, literally: fmod fold into (-pi, pi], sum of
// the four wrapped differences, lround(total / 2pi).
__device__ __forceinline__ double wrap_angle_diff_dev(double d)
{
    const double pi = 3.14159265358979323846;
    const double two_pi = 2.0 * pi;
    d = fmod(d, two_pi);
    if (d <= -pi)
        d += two_pi;
    else if (d > pi)
        d -= two_pi;
    return d;
}

__global__ void plaquette_winding_batch_kernel(const double *__restrict__ th, int64_t n, int32_t *__restrict__ w)
{
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const double t1 = th[4 * q], t2 = th[4 * q + 1], t3 = th[4 * q + 2], t4 = th[4 * q + 3];
    const double total = __dadd_rn(__dadd_rn(__dadd_rn(wrap_angle_diff_dev(__dsub_rn(t2, t1)),
                                                       wrap_angle_diff_dev(__dsub_rn(t3, t2))),
                                             wrap_angle_diff_dev(__dsub_rn(t4, t3))),
                                   wrap_angle_diff_dev(__dsub_rn(t1, t4)));
    w[q] = (int32_t)llround(__ddiv_rn(total, 2.0 * 3.14159265358979323846));
}

// ------------------------------------------------------------ device: Fourier IC spectrum
// FourierIC.hpp:28-116 (SplitMix64 hash, uniform from the top 53 bits,
// Box-Muller, kx unwrapped / ky,kz wrapped, 0 < k^2 <= k_max^2).
__device__ __forceinline__ uint64_t hash_u64_dev(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

__global__ void fourier_spectrum_kernel(double2 *__restrict__ spec, int nx, int ny, int nz, double kmax2,
                                        uint64_t full_seed)
{
    const int nxh = nx / 2 + 1;
    const int64_t total = (int64_t)nxh * ny * nz;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q % nxh);
        const int j = (int)((q / nxh) % ny);
        const int k = (int)(q / ((int64_t)nxh * ny));
        const int kx = i, ky = (j <= ny / 2) ? j : j - ny, kz = (k <= nz / 2) ? k : k - nz;
        const double k2 = (double)(kx * kx + ky * ky + kz * kz);
        double2 out = make_double2(0.0, 0.0);
        if (!(k2 > kmax2 || k2 == 0.0)) {
            const uint64_t key = full_seed ^ ((uint64_t)0 << 60) ^ ((uint64_t)(uint32_t)i << 40) ^
                                 ((uint64_t)(uint32_t)j << 20) ^ (uint64_t)(uint32_t)k;
            const uint64_t h1 = hash_u64_dev(key);
            const uint64_t h2 = hash_u64_dev(key ^ 0x1234567890ABCDEFULL);
            double u1 = ((double)(h1 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
            if (u1 < 1.0e-300) u1 = 1.0e-300;
            const double u2 = ((double)(h2 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
            const double r = sqrt(-2.0 * log(u1));
            double s, c;
            sincos(2.0 * 3.14159265358979323846 * u2, &s, &c);
            out = make_double2(r * c, r * s);
        }
        spec[q] = out;
    }
}

}  // namespace axs

using namespace axs;

extern "C" {

const char *axs_last_error(void) { return g_err; }

int axs_abi_version(void) { return AXS_ABI_VERSION; }

int axs_set_device_wait_polls(uint32_t polls, uint32_t *previous)
{
    const uint32_t prev = g_wait_polls.exchange(polls);
    if (previous) *previous = prev;
    return AXS_OK;
}

const char *axs_status_string(int s)
{
    switch (s) {
    case AXS_OK: return "ok";
    case AXS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case AXS_ERR_UNSUPPORTED: return "unsupported shape or layout";
    case AXS_ERR_ALIGNMENT: return "misaligned pointer or stride";
    case AXS_ERR_WORKSPACE: return "workspace too small";
    case AXS_ERR_CUDA: return "CUDA error";
    case AXS_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
    case AXS_ERR_CAPACITY: return "pierced-plaquette list truncated";
    default: return "unknown status";
    }
}

int axs_background_eval(const axs_background *bg, double tau, axs_background_values *out)
{
    int rc = validate_background(bg);
    if (rc) return rc;
    AXS_REQUIRE(out != nullptr, AXS_ERR_INVALID_ARGUMENT, "null output");
    background_values(*bg, tau, *out);
    return AXS_OK;
}

int axs_background_rhs_coeffs(const axs_background *bg, double tau, axs_rhs_coeffs *out)
{
    int rc = validate_background(bg);
    if (rc) return rc;
    AXS_REQUIRE(out != nullptr, AXS_ERR_INVALID_ARGUMENT, "null output");
    rhs_coeffs(*bg, tau, *out);
    return AXS_OK;
}

int axs_background_tau_from_log_mr_over_h(const axs_background *bg, double l, double *tau)
{
    int rc = validate_background(bg);
    if (rc) return rc;
    AXS_REQUIRE(tau != nullptr, AXS_ERR_INVALID_ARGUMENT, "null output");
    AXS_REQUIRE(bg->kind == AXS_BG_EXPANDING && bg->a_inv != bg->c0, AXS_ERR_INVALID_ARGUMENT,
                "tau_from_log_mr_over_h needs an expanding background with c0 != a_inv");
    *tau = std::exp(l * (bg->a_inv - 1.0) / (bg->a_inv - bg->c0));
    return AXS_OK;
}

double axs_xi_from_comoving_length(double ell, double L, double a_inv, double tau)
{
    const double am1 = a_inv - 1.0;
    return ell / (L * L * L) * (am1 * am1 * am1 / (a_inv * a_inv)) * (tau * tau);
}

double axs_xi_from_plaquette_count(double N_p, double dx, double L, double a_inv, double tau)
{
    return axs_xi_from_comoving_length((2.0 / 3.0) * N_p * dx, L, a_inv, tau);
}

double axs_plaquette_count_for_target_xi(double xi, int N, double L, double a_inv, double tau)
{
    const double am1 = a_inv - 1.0;
    return 3.0 * N * xi * L * L * a_inv * a_inv / (2.0 * am1 * am1 * am1 * tau * tau);
}

int axs_plaquette_winding_batch(const double *theta, int64_t n, int32_t *w, void *stream)
{
    AXS_REQUIRE(n >= 0, AXS_ERR_INVALID_ARGUMENT, "negative count");
    if (n == 0) return AXS_OK;
    AXS_REQUIRE(theta && w, AXS_ERR_INVALID_ARGUMENT, "null pointer");
    const int threads = 256;
    const int64_t blocks = (n + threads - 1) / threads;
    AXS_REQUIRE(blocks < (1LL << 31), AXS_ERR_UNSUPPORTED, "batch too large");
    plaquette_winding_batch_kernel<<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(theta, n, w);
    return launch_status("plaquette_winding_batch");
}

int axs_fourier_spectrum(double *spec, int32_t nx, int32_t ny, int32_t nz, double k_max_cells, uint64_t seed,
                         int32_t comp_seed_offset, void *stream)
{
    AXS_REQUIRE(spec != nullptr, AXS_ERR_INVALID_ARGUMENT, "null spectrum");
    AXS_REQUIRE(nx > 0 && ny > 0 && nz > 0, AXS_ERR_INVALID_ARGUMENT, "empty box");
    const uint64_t full_seed = seed ^ ((uint64_t)(int64_t)comp_seed_offset << 32);
    const int sms = device_sm_count();
    AXS_REQUIRE(sms > 0, AXS_ERR_CUDA, "no CUDA device");
    fourier_spectrum_kernel<<<sms * 8, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<double2 *>(spec), nx, ny,
                                                                        nz, k_max_cells * k_max_cells, full_seed);
    return launch_status("fourier_spectrum");
}

}  // extern "C"
