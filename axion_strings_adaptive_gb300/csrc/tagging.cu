// Refinement tagging on a periodic level: the reference's StringTagger
// (StringTagger.hpp:117-151) plus the n_error_buf buffer AMReX applies before
// clustering, and per-block flags for fixed-size patch clustering.
//
// Per cell (one thread, x fastest): the three plaquette windings at the low
// corner with the string finder's own arithmetic (winding.cuh: single-
// precision phases with a double fallback, so the result is the reference's
// double-atan2 winding bit for bit); when no plaquette is pierced and the
// corresponding threshold is finite, dx^2 |lap psi_i| and dx |grad |psi||
// evaluated with round-to-nearest double operations in the reference's
// expression order (the oracle's FourthOrderDerivatives restatement), so the
// threshold comparisons match the CPU evaluation exactly. The buffer is a
// separable periodic max filter (x, y, z passes); a last pass counts tags and
// flags blocks.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "axs_internal.cuh"
#include "winding.cuh"

namespace axs {

int level_geom(int32_t dtype, int nx, int ny, int nz, LevelGeom &g);
int diag_level_plaquette_tags(const void *state, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g, double dx,
                              uint8_t *tags, axs_diag_result *out, void *scratch, int64_t scratch_bytes,
                              cudaStream_t st);
int64_t diag_scratch_bytes_for(int64_t ncell);

// scratch: [0, 256) tag count and the plaquette pass's result record,
// [256, 256 + tag bytes) buffer pass temporaries, then the plaquette pass's scratch
constexpr int64_t kTagResultOffset = 64;
static int64_t tag_bytes_rounded(int64_t n) { return (n + 255) / 256 * 256; }
static_assert(kTagResultOffset + sizeof(axs_diag_result) <= 256, "tag scratch header");

struct TagGeom {
    int nx, ny, nz, ox, oy;
    int64_t js, ks, cs;
};

struct TagConst {
    double one_over_dx, one_over_dx2, dx2, dx;
    double grad_thr, rad_thr;
    int use_grad, use_rad;
};

__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

template <typename T>
__device__ __forceinline__ int64_t toff(const TagGeom &g, int i, int j, int k)
{
    return (int64_t)(wrapi(i, g.nx) + g.ox) + (int64_t)(wrapi(j, g.ny) + g.oy) * g.js + (int64_t)wrapi(k, g.nz) * g.ks;
}

// GRTeclyn diff2 / diff1 in the oracle's expression order, rounded to T.
__device__ __forceinline__ double tag_diff2(double m2, double m1, double c, double p1, double p2, double s)
{
    const double wf = 8.33333333333333333333e-2, wn = 1.33333333333333333333e+0, wl = 2.5;
    double r = __dmul_rn(-wf, m2);
    r = __dadd_rn(r, __dmul_rn(wn, m1));
    r = __dsub_rn(r, __dmul_rn(wl, c));
    r = __dadd_rn(r, __dmul_rn(wn, p1));
    r = __dsub_rn(r, __dmul_rn(wf, p2));
    return __dmul_rn(r, s);
}

__device__ __forceinline__ double tag_diff1(double m2, double m1, double p1, double p2, double s)
{
    const double wf = 8.33333333333333333333e-2, wn = 6.66666666666666666667e-1;
    double r = __dmul_rn(wf, m2);
    r = __dsub_rn(r, __dmul_rn(wn, m1));
    r = __dadd_rn(r, __dmul_rn(wn, p1));
    r = __dsub_rn(r, __dmul_rn(wf, p2));
    return __dmul_rn(r, s);
}

template <typename T>
__global__ void __launch_bounds__(256) tag_kernel(const T *__restrict__ st, TagGeom g, TagConst q,
                                                   uint8_t *__restrict__ out)
{
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    for (int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; cell < n;
         cell += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(cell % g.nx), j = (int)((cell / g.nx) % g.ny), k = (int)(cell / ((int64_t)g.nx * g.ny));
        const T *p1 = st, *p2 = st + g.cs;
        // corner phases (x, y, z offsets), StringFinder.hpp:45-68 order
        const int64_t o000 = toff<T>(g, i, j, k), o100 = toff<T>(g, i + 1, j, k), o110 = toff<T>(g, i + 1, j + 1, k),
                      o010 = toff<T>(g, i, j + 1, k), o001 = toff<T>(g, i, j, k + 1),
                      o101 = toff<T>(g, i + 1, j, k + 1), o011 = toff<T>(g, i, j + 1, k + 1);
        const int64_t offs[7] = {o000, o100, o110, o010, o001, o101, o011};
        float th[7];
        bool ok = true;
#pragma unroll
        for (int v = 0; v < 7; ++v) {
            const T a = __ldg(p1 + offs[v]), b = __ldg(p2 + offs[v]);
            if constexpr (sizeof(T) == 4) {
                const float m = fmaxf(fabsf(a), fabsf(b));
                ok = ok && m > 1e-30f && m < 1e30f;
            } else {
                const double m = fmax(fabs(a), fabs(b));
                ok = ok && m > 1e-30 && m < 1e30;
            }
            th[v] = atan2f((float)b, (float)a);
        }
        int w[3] = {0, 0, 0};
        if (!(ok && cell_windings_fast(th[0], th[1], th[2], th[3], th[4], th[5], th[6], w))) {
            double d[7];
#pragma unroll
            for (int v = 0; v < 7; ++v) d[v] = atan2((double)__ldg(p2 + offs[v]), (double)__ldg(p1 + offs[v]));
            int ties = 0;
            cell_windings_double(d[0], d[1], d[2], d[3], d[4], d[5], d[6], w, ties);
        }
        uint8_t tag = (w[0] | w[1] | w[2]) != 0;
        if (!tag && q.use_grad) {
            // StringTagger::scalar_laplacian (:159-177): sum over d of diff2 as T, in double
            double lap[2];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const T *p = c == 0 ? p1 : p2;
                double acc = 0.0;
                const int di[3] = {1, 0, 0}, dj[3] = {0, 1, 0}, dk[3] = {0, 0, 1};
#pragma unroll
                for (int dd = 0; dd < 3; ++dd) {
                    const double m2 = __ldg(p + toff<T>(g, i - 2 * di[dd], j - 2 * dj[dd], k - 2 * dk[dd]));
                    const double m1 = __ldg(p + toff<T>(g, i - di[dd], j - dj[dd], k - dk[dd]));
                    const double cc = __ldg(p + o000);
                    const double q1 = __ldg(p + toff<T>(g, i + di[dd], j + dj[dd], k + dk[dd]));
                    const double q2 = __ldg(p + toff<T>(g, i + 2 * di[dd], j + 2 * dj[dd], k + 2 * dk[dd]));
                    acc = __dadd_rn(acc, (double)(T)tag_diff2(m2, m1, cc, q1, q2, q.one_over_dx2));
                }
                lap[c] = acc;
            }
            tag = __dmul_rn(q.dx2, fabs(lap[0])) > q.grad_thr || __dmul_rn(q.dx2, fabs(lap[1])) > q.grad_thr;
        }
        if (!tag && q.use_rad) {
            // StringTagger::radial_gradient_sq (:187-217)
            const double psi1 = __ldg(p1 + o000), psi2 = __ldg(p2 + o000);
            const double psi_sq = __dadd_rn(__dmul_rn(psi1, psi1), __dmul_rn(psi2, psi2));
            double g1 = 0.0, g2 = 0.0, gt = 0.0;
            const int di[3] = {1, 0, 0}, dj[3] = {0, 1, 0}, dk[3] = {0, 0, 1};
#pragma unroll
            for (int dd = 0; dd < 3; ++dd) {
                double dv[2];
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const T *p = c == 0 ? p1 : p2;
                    dv[c] = (double)(T)tag_diff1(__ldg(p + toff<T>(g, i - 2 * di[dd], j - 2 * dj[dd], k - 2 * dk[dd])),
                                                 __ldg(p + toff<T>(g, i - di[dd], j - dj[dd], k - dk[dd])),
                                                 __ldg(p + toff<T>(g, i + di[dd], j + dj[dd], k + dk[dd])),
                                                 __ldg(p + toff<T>(g, i + 2 * di[dd], j + 2 * dj[dd], k + 2 * dk[dd])),
                                                 q.one_over_dx);
                }
                g1 = __dadd_rn(g1, __dmul_rn(dv[0], dv[0]));
                g2 = __dadd_rn(g2, __dmul_rn(dv[1], dv[1]));
                const double dth =
                    psi_sq > 0.0 ? __ddiv_rn(__dsub_rn(__dmul_rn(psi1, dv[1]), __dmul_rn(psi2, dv[0])), psi_sq) : 0.0;
                gt = __dadd_rn(gt, __dmul_rn(dth, dth));
            }
            const double r2 = __dsub_rn(__dadd_rn(g1, g2), __dmul_rn(psi_sq, gt));
            tag = __dmul_rn(q.dx, __dsqrt_rn(r2)) > q.rad_thr;
        }
        out[cell] = tag;
    }
}

// One axis of the periodic cube buffer: out = OR of in over [-nb, nb] along the axis.
__global__ void dilate_axis_kernel(const uint8_t *__restrict__ in, uint8_t *__restrict__ out, int nx, int ny, int nz,
                                   int axis, int nb)
{
    const int64_t n = (int64_t)nx * ny * nz;
    const int len = axis == 0 ? nx : (axis == 1 ? ny : nz);
    const int64_t stride = axis == 0 ? 1 : (axis == 1 ? nx : (int64_t)nx * ny);
    for (int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; cell < n;
         cell += (int64_t)gridDim.x * blockDim.x) {
        const int pos = (int)(axis == 0 ? cell % nx : (axis == 1 ? (cell / nx) % ny : cell / ((int64_t)nx * ny)));
        const int64_t base = cell - (int64_t)pos * stride;
        uint8_t any = 0;
        for (int d = -nb; d <= nb && !any; ++d) {
            int p = (pos + d) % len;
            if (p < 0) p += len;
            any = in[base + (int64_t)p * stride];
        }
        out[cell] = any;
    }
}

// Count tags (integer atomics: deterministic) and flag every block^3 block holding one.
__global__ void tag_count_kernel(const uint8_t *__restrict__ tags, int nx, int ny, int nz, int block,
                                 uint8_t *__restrict__ flags, unsigned long long *__restrict__ count)
{
    const int64_t n = (int64_t)nx * ny * nz;
    const int nbx = block > 0 ? (nx + block - 1) / block : 0, nby = block > 0 ? (ny + block - 1) / block : 0;
    unsigned long long mine = 0;
    for (int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; cell < n;
         cell += (int64_t)gridDim.x * blockDim.x) {
        if (!tags[cell]) continue;
        ++mine;
        if (flags) {
            const int i = (int)(cell % nx), j = (int)((cell / nx) % ny), k = (int)(cell / ((int64_t)nx * ny));
            flags[(i / block) + (int64_t)nbx * ((j / block) + (int64_t)nby * (k / block))] = 1;
        }
    }
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(count, mine);
}

// ---- the buffer on bit-packed tags (nx a multiple of 32): bit b of word w of
// row (y, z) is cell x = 32 w + b. A pass handles 32 cells per word and moves
// an eighth of the byte array's bytes (16 MB for 512^3, held in L2).

// byte tags -> bits
__global__ void tag_pack_kernel(const uint8_t *__restrict__ in, uint32_t *__restrict__ out, int64_t nwords)
{
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < nwords; w += (int64_t)gridDim.x * blockDim.x) {
        const uint4 *p = reinterpret_cast<const uint4 *>(in + 32 * w);
        const uint4 a = p[0], b = p[1];
        const uint32_t v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        uint32_t bits = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
            for (int k = 0; k < 4; ++k) bits |= (uint32_t)(((v[q] >> (8 * k)) & 0xffu) != 0) << (4 * q + k);
        out[w] = bits;
    }
}

__device__ __forceinline__ int wrap_small(int i, int n)
{
    while (i < 0) i += n;
    while (i >= n) i -= n;
    return i;
}

// x: OR over cells x - nb .. x + nb of the row (periodic over W words)
__global__ void tag_dilate_x_bits_kernel(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, int W,
                                         int64_t nwords, int nb)
{
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < nwords; w += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = w / W;
        const int i = (int)(w - row * W);
        const uint32_t *r = in + row * W;
        uint32_t acc = r[i];
        for (int d = 1; d <= nb; ++d) {
            const int q = d >> 5, sh = d & 31;
            // cells x + d from words i + q, i + q + 1; cells x - d from words i - q - 1, i - q
            acc |= __funnelshift_r(r[wrap_small(i + q, W)], r[wrap_small(i + q + 1, W)], sh) |
                   __funnelshift_l(r[wrap_small(i - q - 1, W)], r[wrap_small(i - q, W)], sh);
        }
        out[w] = acc;
    }
}

// y or z: OR over rows pos - nb .. pos + nb along an axis of len rows, stride words apart
__global__ void tag_dilate_rows_bits_kernel(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                                            int64_t nwords, int64_t stride, int len, int nb)
{
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < nwords; w += (int64_t)gridDim.x * blockDim.x) {
        const int pos = (int)((w / stride) % len);
        const int64_t base = w - (int64_t)pos * stride;
        uint32_t acc = 0;
        for (int d = -nb; d <= nb; ++d) acc |= in[base + (int64_t)wrap_small(pos + d, len) * stride];
        out[w] = acc;
    }
}

// bits -> byte tags (when out is given), the tag count and the block flags
__global__ void tag_unpack_count_kernel(const uint32_t *__restrict__ bits, uint8_t *__restrict__ out, int W, int ny,
                                        int nz, int block, uint8_t *__restrict__ flags,
                                        unsigned long long *__restrict__ count, int64_t nwords)
{
    const int nbx = block > 0 ? (32 * W + block - 1) / block : 0, nby = block > 0 ? (ny + block - 1) / block : 0;
    unsigned long long mine = 0;
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < nwords; w += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t b = bits[w];
        if (out != nullptr) {
            uint32_t v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const uint32_t nib = (b >> (4 * q)) & 15u;  // cells 4q .. 4q + 3 -> bytes 0 .. 3
                v[q] = (nib & 1u) | ((nib & 2u) << 7) | ((nib & 4u) << 14) | ((nib & 8u) << 21);
            }
            uint4 *o = reinterpret_cast<uint4 *>(out + 32 * w);
            o[0] = make_uint4(v[0], v[1], v[2], v[3]);
            o[1] = make_uint4(v[4], v[5], v[6], v[7]);
        }
        mine += __popc(b);
        if (flags != nullptr && b != 0) {
            const int64_t row = w / W;
            const int i = (int)(w - row * W), j = (int)(row % ny), k = (int)(row / ny);
            const int64_t fb = (int64_t)nbx * ((j / block) + (int64_t)nby * (k / block));
            uint32_t m = b;
            while (m) {
                const int bx = (32 * i + __ffs(m) - 1) / block;
                flags[bx + fb] = 1;
                const int next = (bx + 1) * block - 32 * i;  // first bit of the next block
                m = next >= 32 ? 0u : (m & (~0u << next));
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(count, mine);
}

static int tag_grid(int64_t n)
{
    const int sms = device_sm_count() > 0 ? device_sm_count() : 148;
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 8));
}

}  // namespace axs

using namespace axs;

extern "C" {

int axs_tag_scratch_bytes(int32_t nx, int32_t ny, int32_t nz, int64_t *bytes)
{
    AXS_REQUIRE(bytes != nullptr && nx > 0 && ny > 0 && nz > 0, AXS_ERR_INVALID_ARGUMENT, "bad arguments");
    const int64_t n = (int64_t)nx * ny * nz;
    *bytes = 256 + tag_bytes_rounded(n) + diag_scratch_bytes_for(n);
    return AXS_OK;
}

int axs_level_tag_cells(const axs_level *lv, const axs_tag_params *p, uint8_t *tags_dev, uint8_t *block_flags_dev,
                        int64_t *n_tagged_dev, void *scratch, int64_t scratch_bytes, void *stream)
{
    AXS_REQUIRE(lv != nullptr && lv->state != nullptr && p != nullptr && tags_dev != nullptr,
                AXS_ERR_INVALID_ARGUMENT, "null argument");
    LevelGeom lg;
    int rc = level_geom(lv->dtype, lv->nx, lv->ny, lv->nz, lg);
    if (rc) return rc;
    AXS_REQUIRE(p->dx > 0.0, AXS_ERR_INVALID_ARGUMENT, "dx must be positive");
    AXS_REQUIRE(lv->ny >= 2 && lv->nz >= 2, AXS_ERR_UNSUPPORTED, "tagging needs ny, nz >= 2");
    AXS_REQUIRE(p->n_error_buf >= 0 && p->block >= 0, AXS_ERR_INVALID_ARGUMENT, "negative buffer or block size");
    AXS_REQUIRE(p->n_error_buf <= 64, AXS_ERR_UNSUPPORTED, "n_error_buf %d too large", p->n_error_buf);
    AXS_REQUIRE(p->block == 0 || block_flags_dev != nullptr, AXS_ERR_INVALID_ARGUMENT, "null block flags");
    int64_t need = 0;
    axs_tag_scratch_bytes(lv->nx, lv->ny, lv->nz, &need);
    AXS_REQUIRE(scratch != nullptr && scratch_bytes >= need, AXS_ERR_WORKSPACE, "tag scratch too small (%lld < %lld)",
                (long long)scratch_bytes, (long long)need);
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t n = (int64_t)lv->nx * lv->ny * lv->nz;
    auto *count = static_cast<unsigned long long *>(scratch);
    uint8_t *tmp = static_cast<uint8_t *>(scratch) + 256;
    TagGeom g{lv->nx, lv->ny, lv->nz, lg.ox, lg.oy, lg.js, lg.ks, lg.cs};
    TagConst q{};
    const double dxr = lv->dtype == AXS_F32 ? (double)(float)p->dx : p->dx;  // m_dx is amrex::Real
    q.dx = dxr;
    q.dx2 = lv->dtype == AXS_F32 ? (double)((float)dxr * (float)dxr) : dxr * dxr;
    q.one_over_dx = 1.0 / p->dx;
    q.one_over_dx2 = 1.0 / (p->dx * p->dx);
    q.grad_thr = p->gradient_threshold;
    q.rad_thr = p->radial_gradient_threshold;
    // a threshold at DBL_MAX or above ("off" in the reference) can only be crossed
    // by an overflowed value; the criterion is skipped
    q.use_grad = p->gradient_threshold < DBL_MAX;
    q.use_rad = p->radial_gradient_threshold < DBL_MAX;
    const int grid = tag_grid(n);
    uint8_t *first = p->n_error_buf > 0 ? tmp : tags_dev;
    if (!q.use_grad && !q.use_rad) {
        // the plaquette criterion alone (the reference's default): the string
        // finder's tiled pass, one phase per vertex instead of seven per cell
        char *base = static_cast<char *>(scratch);
        const int64_t off = 256 + tag_bytes_rounded(n);
        auto *res = reinterpret_cast<axs_diag_result *>(base + kTagResultOffset);
        if ((rc = diag_level_plaquette_tags(lv->state, lv->dtype, lv->nx, lv->ny, lv->nz, lg, p->dx, first, res,
                                            base + off, scratch_bytes - off, st)))
            return rc;
    } else {
        if (lv->dtype == AXS_F32)
            tag_kernel<float><<<grid, 256, 0, st>>>(static_cast<const float *>(lv->state), g, q, first);
        else
            tag_kernel<double><<<grid, 256, 0, st>>>(static_cast<const double *>(lv->state), g, q, first);
        if ((rc = launch_status("tag cells"))) return rc;
    }
    // the buffer and the count on bit-packed tags: rows of whole words, and
    // 16-byte aligned byte arrays for the vector loads and stores
    const bool bits = lv->nx % 32 == 0 && ((uintptr_t)tags_dev % 16) == 0 && ((uintptr_t)tmp % 16) == 0;
    const int64_t nwords = n / 32;
    const int wgrid = tag_grid(nwords);
    const int W = lv->nx / 32;
    if (bits) {
        AXS_CUDA_CHECK(cudaMemsetAsync(count, 0, sizeof(unsigned long long), st));
        if (p->block > 0) {
            const int64_t nb = (int64_t)((lv->nx + p->block - 1) / p->block) * ((lv->ny + p->block - 1) / p->block) *
                               ((lv->nz + p->block - 1) / p->block);
            AXS_CUDA_CHECK(cudaMemsetAsync(block_flags_dev, 0, (size_t)nb, st));
        }
        auto *tmp_bits = reinterpret_cast<uint32_t *>(tmp);
        if (p->n_error_buf > 0) {
            // bytes in tmp -> bits A (in the output array, not yet written) -> x -> B (tmp) -> y -> A -> z -> B
            auto *a = reinterpret_cast<uint32_t *>(tags_dev);
            tag_pack_kernel<<<wgrid, 256, 0, st>>>(tmp, a, nwords);
            tag_dilate_x_bits_kernel<<<wgrid, 256, 0, st>>>(a, tmp_bits, W, nwords, p->n_error_buf);
            tag_dilate_rows_bits_kernel<<<wgrid, 256, 0, st>>>(tmp_bits, a, nwords, W, lv->ny, p->n_error_buf);
            tag_dilate_rows_bits_kernel<<<wgrid, 256, 0, st>>>(a, tmp_bits, nwords, (int64_t)W * lv->ny, lv->nz,
                                                              p->n_error_buf);
            tag_unpack_count_kernel<<<wgrid, 256, 0, st>>>(tmp_bits, tags_dev, W, lv->ny, lv->nz, p->block,
                                                          p->block > 0 ? block_flags_dev : nullptr, count, nwords);
        } else {
            tag_pack_kernel<<<wgrid, 256, 0, st>>>(tags_dev, tmp_bits, nwords);
            tag_unpack_count_kernel<<<wgrid, 256, 0, st>>>(tmp_bits, nullptr, W, lv->ny, lv->nz, p->block,
                                                          p->block > 0 ? block_flags_dev : nullptr, count, nwords);
        }
        if ((rc = launch_status("tag buffer and count"))) return rc;
        if (n_tagged_dev)
            AXS_CUDA_CHECK(cudaMemcpyAsync(n_tagged_dev, count, sizeof(int64_t), cudaMemcpyDeviceToDevice, st));
        return AXS_OK;
    }
    if (p->n_error_buf > 0) {
        dilate_axis_kernel<<<grid, 256, 0, st>>>(tmp, tags_dev, lv->nx, lv->ny, lv->nz, 0, p->n_error_buf);
        dilate_axis_kernel<<<grid, 256, 0, st>>>(tags_dev, tmp, lv->nx, lv->ny, lv->nz, 1, p->n_error_buf);
        dilate_axis_kernel<<<grid, 256, 0, st>>>(tmp, tags_dev, lv->nx, lv->ny, lv->nz, 2, p->n_error_buf);
        if ((rc = launch_status("tag buffer"))) return rc;
    }
    if (n_tagged_dev != nullptr || p->block > 0) {
        AXS_CUDA_CHECK(cudaMemsetAsync(count, 0, sizeof(unsigned long long), st));
        if (p->block > 0) {
            const int64_t nb = (int64_t)((lv->nx + p->block - 1) / p->block) * ((lv->ny + p->block - 1) / p->block) *
                               ((lv->nz + p->block - 1) / p->block);
            AXS_CUDA_CHECK(cudaMemsetAsync(block_flags_dev, 0, (size_t)nb, st));
        }
        tag_count_kernel<<<grid, 256, 0, st>>>(tags_dev, lv->nx, lv->ny, lv->nz, p->block,
                                                p->block > 0 ? block_flags_dev : nullptr, count);
        if ((rc = launch_status("tag count"))) return rc;
        if (n_tagged_dev)
            AXS_CUDA_CHECK(cudaMemcpyAsync(n_tagged_dev, count, sizeof(int64_t), cudaMemcpyDeviceToDevice, st));
    }
    return AXS_OK;
}

}  // extern "C"
