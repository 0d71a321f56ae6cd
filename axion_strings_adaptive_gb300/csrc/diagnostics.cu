// Fused diagnostics pass: plaquette windings + pierced list (string finder),
// the 14 screened/unscreened energy sums, and gamma^2 v^2 at pierced corners,
// in one sweep over the valid cells.
//
// Reference: StringFinder.hpp:45-122, PlaquetteWinding.hpp:24-51,
// EnergyKernel.hpp:106-233, Energy.hpp:64-190, Masking.hpp:75-93,
// VelocityKernel.hpp:37-141, Velocity.hpp:62-78.
//
// Windings follow the reference literally: double atan2 of the (double-cast)
// field at each corner, fmod fold into (-pi, pi], lround of the sum / 2 pi.
// Edges whose |dtheta| lies within 1e-12 of pi are counted as "near ties":
// only there could a different correctly-rounded-to-1-ulp atan2 flip a fold.
// All per-cell energy/velocity arithmetic is FP64 whatever the field
// precision; sums go per thread -> warp shuffle -> block -> per-block partial
// in scratch -> a single-block finalize in a fixed order (deterministic, no
// floating-point atomics).
#include <climits>
#include <cmath>
#include <mutex>

#include <algorithm>
#include <type_traits>

#include "axs_internal.cuh"
#include "winding.cuh"

namespace axs {

struct DiagView {
    const void *data;
    int32_t dtype;
    int nx, ny, nz;
    int ox, oy, oz;          // offset of valid cell (0,0,0) in elements along each axis
    int wx, wy, wz;          // 1: wrap indices periodically on that axis; 0: read ghosts
    int64_t js, ks, cs;
};

struct DiagPartial {
    double e[14];
    double vsum;
    long long cnt[4];  // n_p_plain, n_p_weighted, vel_count, near_tie
    double pad;
};
static_assert(sizeof(DiagPartial) == 160, "partial layout");

constexpr int kDiagThreads = 256;

struct DiagConst {
    double one_over_dx, R, lambda, RpR, m_r, threshold;
    double R2, inv_R, inv_R2, inv_R4;
    double vel_a, vel_b, vel_c;  // gamma^2 v^2 = |phi'|^2 vel_a (1 - vel_b |phi|^2) - vel_c (phi . phi')^2
    int scheme;
    int want_energy, want_plaq, want_vel;
    // single-precision copies for the per_cell_fp32 variant
    float f_one_over_dx, f_R2, f_inv_R, f_inv_R2, f_inv_R4, f_lambda, f_RpR, f_threshold;
    float f_vel_a, f_vel_b, f_vel_c;
};

template <typename T>
__device__ __forceinline__ int64_t view_off(const DiagView &v, int c, int i, int j, int k)
{
    if (v.wx) i = (i % v.nx + v.nx) % v.nx;
    if (v.wy) j = (j % v.ny + v.ny) % v.ny;
    if (v.wz) k = (k % v.nz + v.nz) % v.nz;
    return c * v.cs + (int64_t)(i + v.ox) + (int64_t)(j + v.oy) * v.js + (int64_t)(k + v.oz) * v.ks;
}

template <typename T>
__device__ __forceinline__ double ld(const DiagView &v, int c, int i, int j, int k)
{
    return (double)__ldg(static_cast<const T *>(v.data) + view_off<T>(v, c, i, j, k));
}

// GRTeclyn diff1 (centred 4th order: weights 1/12, 2/3, times 1/dx) from
// the four neighbours, rounded to the field precision as d1_scalar returns
// amrex::Real. FP32 fields: the reference's expression order with explicit
// round-to-nearest double operations, since a fused multiply-add could move
// the rounded float by one ulp. FP64 fields: contraction allowed.
template <typename T>
__device__ __forceinline__ double diff1_vals(double m2, double m1, double p1, double p2, double inv_dx)
{
    const double wf = 8.33333333333333333333e-2, wn = 6.66666666666666666667e-1;
    if constexpr (sizeof(T) == 4) {
        double r = __dmul_rn(wf, m2);
        r = __dsub_rn(r, __dmul_rn(wn, m1));
        r = __dadd_rn(r, __dmul_rn(wn, p1));
        r = __dsub_rn(r, __dmul_rn(wf, p2));
        return (double)(float)__dmul_rn(r, inv_dx);
    } else {
        return (wf * m2 - wn * m1 + wn * p1 - wf * p2) * inv_dx;
    }
}

// float -> double without the conversion unit: GB300 issues FP32 <-> FP64
// conversions at its FP64 rate (1/64 of FP32), and the FP64 per-cell pass
// converts every stencil tap. Normal numbers and zeros by integer operations
// (the same double the conversion gives), the rest by the conversion.
__device__ __forceinline__ double f2d_exact(float x)
{
    const unsigned u = __float_as_uint(x), e = (u >> 23) & 0xffu;
    const unsigned long long sgn = (unsigned long long)(u >> 31) << 63;
    if (e - 1u < 254u)
        return __longlong_as_double(
            (long long)(sgn | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
    if ((u << 1) == 0u) return __longlong_as_double((long long)sgn);
    return (double)x;
}

// a field value as double: FP32 widened by f2d_exact, FP64 as it is
template <typename T> __device__ __forceinline__ double widen(T x)
{
    if constexpr (sizeof(T) == 4)
        return f2d_exact(x);
    else
        return x;
}

// diff1_vals for FP32 fields from float taps: the same operations; r32 is the
// rounded float the reference squares, the return value its double.
__device__ __forceinline__ double diff1_f32(float m2, float m1, float p1, float p2, double inv_dx, float &r32)
{
    const double wf = 8.33333333333333333333e-2, wn = 6.66666666666666666667e-1;
    double r = __dmul_rn(wf, f2d_exact(m2));
    r = __dsub_rn(r, __dmul_rn(wn, f2d_exact(m1)));
    r = __dadd_rn(r, __dmul_rn(wn, f2d_exact(p1)));
    r = __dsub_rn(r, __dmul_rn(wf, f2d_exact(p2)));
    r32 = __double2float_rn(__dmul_rn(r, inv_dx));
    return f2d_exact(r32);
}

// The seven per-cell energy terms (EnergyKernel.hpp:130-190) and the masking
// weight (Masking.hpp:75-93) from psi, Pi and the six diff1 values, in math
// type M: double as the reference computes them, or float for the
// per_cell_fp32 variant.
template <typename M> struct CellConst {
    M R2, inv_R, inv_R2, inv_R4, lambda, RpR, threshold;
};

// gt: the diff1 values in the field precision (the reference squares them there)
template <typename M, typename T>
__device__ __forceinline__ void cell_energy_g(const CellConst<M> &k, int scheme, M psi1, M psi2, M Pi1, M Pi2,
                                              const M (&g)[2][3], const T (&gt)[2][3], M (&term)[6], M &wgt)
{
    const M psi_sq = psi1 * psi1 + psi2 * psi2;
    M g1sq = 0, g2sq = 0, cross2 = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if constexpr (sizeof(M) == 8 && sizeof(T) == 4) {
            // the reference squares the float diff1 values in float
            g1sq += f2d_exact(gt[0][d] * gt[0][d]);
            g2sq += f2d_exact(gt[1][d] * gt[1][d]);
        } else if constexpr (sizeof(M) == 8) {
            g1sq += (M)(gt[0][d] * gt[0][d]);
            g2sq += (M)(gt[1][d] * gt[1][d]);
        } else {
            g1sq += g[0][d] * g[0][d];
            g2sq += g[1][d] * g[1][d];
        }
        const M cr = psi1 * g[1][d] - psi2 * g[0][d];
        cross2 += cr * cr;
    }
    const M inv_psq = psi_sq > M(0) ? M(1) / psi_sq : M(0);
    const M gtsq = cross2 * inv_psq * inv_psq;
    const M c1 = Pi1 - k.RpR * psi1, c2 = Pi2 - k.RpR * psi2;
    const M dsq = psi_sq - k.R2;
    const M pot = M(0.25) * k.lambda * dsq * dsq;
    term[0] = (c1 * c1 + c2 * c2 + (g1sq + g2sq) + pot) * k.inv_R4;  // rho
    const M thp = (psi1 * Pi2 - Pi1 * psi2) * inv_psq;
    term[1] = thp * thp * k.inv_R2;                                  // 1/2 (sqrt(2) theta'/R)^2
    term[2] = gtsq * k.inv_R2;                                       // 1/2 sqrt(2)^2 |grad theta|^2 / R^2
    const M rdot = psi1 * c1 + psi2 * c2;
    term[3] = rdot * rdot * inv_psq * k.inv_R4;                      // radial kinetic
    term[4] = (g1sq + g2sq - psi_sq * gtsq) * k.inv_R4;              // radial gradient
    term[5] = pot * k.inv_R4;                                        // radial mass
    wgt = M(1);
    if (scheme != AXS_MASK_NONE) {
        const M mod = sqrt(psi_sq) * k.inv_R;
        if (scheme == AXS_MASK_B) {
            wgt = (mod >= k.threshold) ? M(1) : M(0);
        } else {
            const M f = M(1) + (mod - M(1)) * M(0.70710678118654752440);  // 1 + r / f_a
            wgt = f * f;
        }
    }
}

template <typename M, typename T>
__device__ __forceinline__ void cell_energy(const CellConst<M> &k, int scheme, M psi1, M psi2, M Pi1, M Pi2,
                                            const M (&g)[2][3], M (&term)[6], M &wgt)
{
    T gt[2][3];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) gt[c][d] = (T)g[c][d];
    cell_energy_g<M, T>(k, scheme, psi1, psi2, Pi1, Pi2, g, gt, term, wgt);
}

// Tiled diagnostics pass. A block owns a DTX x DTY tile of cells and marches
// in z over a chunk. Shared memory holds psi1/psi2 of six planes (tile plus a
// 2-cell halo: the five of the gradient stencil and one in flight), Pi1/Pi2 of
// three vertex planes ((DTX+1) x (DTY+1) vertices: z, z+1 and one in flight),
// and for the two vertex planes z and z+1 the single-precision phases and
// gamma^2 v^2, each computed once per vertex. Planes arrive by element-wise
// cp.async one plane ahead of their use, so their latency overlaps the
// current plane's work. Plane loads use element offsets precomputed per work
// item, so the march needs no index division.
constexpr int DTX = 32, DTY = 8, DHX = DTX + 4, DHY = DTY + 4, DVX = DTX + 1, DVY = DTY + 1;
static_assert(DTX * DTY == kDiagThreads, "one cell per thread");
constexpr int kPsiPts = DHX * DHY, kVtxPts = DVX * DVY;
constexpr int kPsiPer = (2 * kPsiPts + kDiagThreads - 1) / kDiagThreads;  // psi loads per thread per plane
constexpr int kPiPer = (2 * kVtxPts + kDiagThreads - 1) / kDiagThreads;   // Pi loads per thread per plane
constexpr int kVtxPer = (kVtxPts + kDiagThreads - 1) / kDiagThreads;      // vertices per thread per plane

// Ring depths for one block barrier per plane: a plane's loads are issued
// before that barrier, so a slot may be refilled only once every thread is
// past the plane that last read it (psi: the 5-plane stencil plus two;
// Pi: read at its vertex plane and again at its cell plane, plus two).
// Vertex planes are computed one plane ahead into a third slot.
constexpr int kPsiSlots = 7, kPiSlots = 5, kVtxSlots = 3;
// pierced plaquettes buffered per block; flushed to the global list with one
// atomic once a plane could overflow it (at most 3 entries per cell)
constexpr int kListBuf = 1536, kListFlushAt = kListBuf - 3 * kDiagThreads;
template <typename T, bool FAST> struct DiagSmem {
    long long lbuf[kListBuf];
    T ps[kPsiSlots][2][DHY][DHX];
    T pi[kPiSlots][2][DVY][DVX];
    typename std::conditional<FAST, float, double>::type gv[kVtxSlots][DVY][DVX];
    float th[kVtxSlots][DVY][DVX];
    unsigned char ok[kVtxSlots][DVY][DVX];
};

__device__ __forceinline__ int wrap_or_self(int i, int n, int wrap) { return wrap ? (i % n + n) % n : i; }

template <typename T, bool FAST>
__global__ void __launch_bounds__(kDiagThreads, 2) diag_kernel(const DiagView v, const DiagConst q,
                                                               const uint8_t *__restrict__ mask,
                                                               DiagPartial *__restrict__ partials,
                                                               unsigned long long *__restrict__ list_counter,
                                                               long long *__restrict__ list, long long capacity,
                                                               int tiles_x, int ntiles, int zchunk, long long n_items,
                                                               long long items_per_box, int64_t box_stride,
                                                               uint8_t *__restrict__ tags)
{
    extern __shared__ __align__(16) unsigned char diag_smem_raw[];
    DiagSmem<T, FAST> &sm = *reinterpret_cast<DiagSmem<T, FAST> *>(diag_smem_raw);
    __shared__ int lcount, flush_n;
    __shared__ unsigned long long flush_base;
    const int64_t box_cells = (int64_t)v.nx * v.ny * v.nz;

    double e[14];
#pragma unroll
    for (int s = 0; s < 14; ++s) e[s] = 0.0;
    // per_cell_fp32: one work item's cells are summed in float, then added to e
    // with compensation (Neumaier) for the 13 real-valued sums; the cell count is exact
    float ef[FAST ? 14 : 1], ec[FAST ? 13 : 1];
#pragma unroll
    for (int s = 0; s < (FAST ? 14 : 1); ++s) ef[s] = 0.f;
#pragma unroll
    for (int s = 0; s < (FAST ? 13 : 1); ++s) ec[s] = 0.f;
    auto csum = [](float &sum, float &comp, float x) {
        const float t = sum + x;
        comp += fabsf(sum) >= fabsf(x) ? (sum - t) + x : (x - t) + sum;
        sum = t;
    };
    const CellConst<double> kd{q.R2, q.inv_R, q.inv_R2, q.inv_R4, q.lambda, q.RpR, q.threshold};
    const CellConst<float> kf{q.f_R2, q.f_inv_R, q.f_inv_R2, q.f_inv_R4, q.f_lambda, q.f_RpR, q.f_threshold};
    double vsum = 0.0;
    long long cnt[4] = {0, 0, 0, 0};

    const int tid = threadIdx.x;
    const int lx = tid % DTX, ly = tid / DTX;
    if (tid == 0) lcount = 0;
    int warp_end = 0;  // end of this warp's last append to lbuf (lane-uniform)
    // move the buffered pierced plaquettes to the global list (called by the whole block)
    auto flush = [&]() {
        if (tid == 0) {
            const int nb = lcount;
            flush_n = nb;
            flush_base = nb ? atomicAdd(list_counter, (unsigned long long)nb) : 0ull;
            lcount = 0;
        }
        __syncthreads();
        const int nb = flush_n;
        const unsigned long long b0 = flush_base;
        for (int i = tid; i < nb; i += kDiagThreads)
            if (b0 + i < (unsigned long long)capacity) list[b0 + i] = sm.lbuf[i];
        __syncthreads();
        warp_end = 0;
    };

    for (long long item = blockIdx.x; item < n_items; item += gridDim.x) {
        // boxes of one batch share the view's geometry and sit box_stride apart
        const long long qbox = item / items_per_box, box_item = item % items_per_box;
        const T *__restrict__ base = static_cast<const T *>(v.data) + qbox * box_stride;
        const int tile = (int)(box_item % ntiles);
        const int chunk = (int)(box_item / ntiles);
        const int x0 = (tile % tiles_x) * DTX, y0 = (tile / tiles_x) * DTY;
        const int za = chunk * zchunk, len = min(zchunk, v.nz - za);

        // ---- per-item load plan: in-plane element offsets (wrapped or ghost) ----
        int64_t psi_off[kPsiPer];  // component + in-plane element offset
        bool psi_ok[kPsiPer];
#pragma unroll
        for (int u = 0; u < kPsiPer; ++u) {
            const int idx = tid + u * kDiagThreads;
            const int c = idx / kPsiPts, r = idx % kPsiPts;
            const int xx = x0 - 2 + r % DHX, yy = y0 - 2 + r / DHX;
            psi_ok[u] = idx < 2 * kPsiPts && xx < v.nx + 2 && yy < v.ny + 2 && (v.wx || (xx >= -v.ox && xx < v.nx + v.ox)) &&
                        (v.wy || (yy >= -v.oy && yy < v.ny + v.oy));
            psi_off[u] = c * v.cs + (int64_t)(wrap_or_self(xx, v.nx, v.wx) + v.ox) +
                         (int64_t)(wrap_or_self(yy, v.ny, v.wy) + v.oy) * v.js;
        }
        int64_t pi_off[kPiPer];
        bool pi_ok[kPiPer];
#pragma unroll
        for (int u = 0; u < kPiPer; ++u) {
            const int idx = tid + u * kDiagThreads;
            const int c = idx / kVtxPts, r = idx % kVtxPts;
            const int xx = x0 + r % DVX, yy = y0 + r / DVX;
            pi_ok[u] = idx < 2 * kVtxPts && xx <= v.nx && yy <= v.ny && (v.wx || xx < v.nx + v.ox) &&
                       (v.wy || yy < v.ny + v.oy);
            pi_off[u] = (2 + c) * v.cs + (int64_t)(wrap_or_self(xx, v.nx, v.wx) + v.ox) +
                        (int64_t)(wrap_or_self(yy, v.ny, v.wy) + v.oy) * v.js;
        }
        auto plane_off = [&](int z, bool &zin) -> int64_t {
            zin = v.wz || (z >= -v.oz && z < v.nz + v.oz);
            return (int64_t)(wrap_or_self(z, v.nz, v.wz) + v.oz) * v.ks;
        };
        // psi of plane z (za - 2 <= z <= za + len + 1) sits in slot (z - za + 2) mod 6,
        // Pi of vertex plane z (za <= z <= za + len) in slot (z - za) mod 3
        auto psi_slot = [&](int z) { return (z - za + 2) % kPsiSlots; };
        auto load_psi = [&](int z) {
            bool zin;
            const int64_t po = plane_off(z, zin);
            T *dst = &sm.ps[psi_slot(z)][0][0][0];
#pragma unroll
            for (int u = 0; u < kPsiPer; ++u) {
                const int idx = tid + u * kDiagThreads;
                if (idx < 2 * kPsiPts) cp_async_elem(dst + idx, base + psi_off[u] + po, zin && psi_ok[u], base);
            }
        };
        auto load_pi = [&](int z) {
            if (!q.want_energy && !q.want_vel) return;  // the string finder alone reads psi only
            bool zin;
            const int64_t po = plane_off(z, zin);
            T *pdst = &sm.pi[(z - za) % kPiSlots][0][0][0];
#pragma unroll
            for (int u = 0; u < kPiPer; ++u) {
                const int idx = tid + u * kDiagThreads;
                if (idx < 2 * kVtxPts) cp_async_elem(pdst + idx, base + pi_off[u] + po, zin && pi_ok[u], base);
            }
        };
        // vertex plane z: phases and gamma^2 v^2 from psi and Pi already in shared memory
        auto vertex_plane = [&](int z) {
            const int ts = (z - za) % kVtxSlots;
            const int ps_ = (z - za) % kPiSlots;
            const int slot = psi_slot(z);
#pragma unroll
            for (int u = 0; u < kVtxPer; ++u) {
                const int idx = tid + u * kDiagThreads;
                if (idx >= kVtxPts) break;
                const int vy = idx / DVX, vx = idx % DVX;
                const T a = sm.ps[slot][0][vy + 2][vx + 2], b = sm.ps[slot][1][vy + 2][vx + 2];
                // float conversion keeps the angle to ~1e-7 only away from under/overflow
                if constexpr (sizeof(T) == 4) {
                    const float m = fmaxf(fabsf(a), fabsf(b));
                    sm.ok[ts][vy][vx] = (m > 1e-30f && m < 1e30f) ? 1 : 0;
                } else {
                    const double m = fmax(fabs(a), fabs(b));
                    sm.ok[ts][vy][vx] = (m > 1e-30 && m < 1e30) ? 1 : 0;
                }
                sm.th[ts][vy][vx] = atan2f((float)b, (float)a);
                if (q.want_vel && FAST) {
                    const float psi1 = a, psi2 = b, Pi1 = sm.pi[ps_][0][vy][vx], Pi2 = sm.pi[ps_][1][vy][vx];
                    const float phi1 = psi1 * q.f_inv_R, phi2 = psi2 * q.f_inv_R;
                    const float pd1 = (Pi1 - q.f_RpR * psi1) * q.f_inv_R2, pd2 = (Pi2 - q.f_RpR * psi2) * q.f_inv_R2;
                    const float phi_sq = phi1 * phi1 + phi2 * phi2;
                    const float pd_sq = pd1 * pd1 + pd2 * pd2;
                    const float re = phi1 * pd1 + phi2 * pd2;
                    sm.gv[ts][vy][vx] = pd_sq * q.f_vel_a * (1.f - q.f_vel_b * phi_sq) - q.f_vel_c * re * re;
                } else if (q.want_vel) {
                    const double psi1 = widen(a), psi2 = widen(b), Pi1 = widen(sm.pi[ps_][0][vy][vx]),
                                 Pi2 = widen(sm.pi[ps_][1][vy][vx]);
                    const double phi1 = psi1 * q.inv_R, phi2 = psi2 * q.inv_R;
                    const double pd1 = (Pi1 - q.RpR * psi1) * q.inv_R2, pd2 = (Pi2 - q.RpR * psi2) * q.inv_R2;
                    const double phi_sq = phi1 * phi1 + phi2 * phi2;
                    const double pd_sq = pd1 * pd1 + pd2 * pd2;
                    const double re = phi1 * pd1 + phi2 * pd2;
                    // Velocity.hpp:62-78 with the constant prefactors folded on the host
                    sm.gv[ts][vy][vx] = pd_sq * q.vel_a * (1.0 - q.vel_b * phi_sq) - q.vel_c * re * re;
                }
            }
        };

        // prologue: psi of za-2 .. za+2 and Pi of za .. za+2 (one group), then the
        // first two vertex planes. Vertex planes run za .. za+len, psi planes
        // za-2 .. za+len+1.
        for (int p = -2; p <= 2; ++p) load_psi(za + p);
        load_pi(za);
        load_pi(za + 1);
        if (len >= 2) load_pi(za + 2);
        cp_async_commit();
        cp_async_wait<0>();
        __syncthreads();
        vertex_plane(za);
        vertex_plane(za + 1);

        for (int m = 0; m < len; ++m) {
            const int z = za + m;
            // one plane ahead: psi(z + 3) for the next plane's stencil and vertex
            // plane, Pi(z + 3) for its vertex plane. Their slots were last read
            // two planes back, before the previous plane's barrier.
            if (m + 1 < len) load_psi(z + 3);
            if (m + 3 <= len) load_pi(z + 3);
            cp_async_commit();
            cp_async_wait<1>();  // everything but this plane's group: psi(z + 2), Pi(z + 2)
            // the plane's one barrier: its psi / Pi and vertex planes z, z + 1 are
            // visible, every thread is done with plane z - 1, and the block learns
            // whether the pierced buffer could overflow during this plane
            if (__syncthreads_or(warp_end > kListFlushAt)) flush();
            // vertex plane z + 2 for the next plane, into the slot plane z - 1 read
            if (m + 2 <= len) vertex_plane(z + 2);

            const int x = x0 + lx, y = y0 + ly;
            const int64_t cell = qbox * box_cells + (int64_t)x + (int64_t)v.nx * ((int64_t)y + (int64_t)v.ny * z);
            const bool in = x < v.nx && y < v.ny && (mask == nullptr || mask[cell] != 0);
            int w[3] = {0, 0, 0};
            if (in) {
                const int s0 = (m + 2) % kPsiSlots;
                const int sm1 = (m + 1) % kPsiSlots, sp1 = (m + 3) % kPsiSlots, sm2 = m % kPsiSlots,
                          sp2 = (m + 4) % kPsiSlots;
                const int t0 = m % kVtxSlots, t1 = (m + 1) % kVtxSlots, tp = m % kPiSlots;
                const int hx = lx + 2, hy = ly + 2;
                if (q.want_energy) {
                    const T p1 = sm.ps[s0][0][hy][hx], p2 = sm.ps[s0][1][hy][hx];
                    const T q1 = sm.pi[tp][0][ly][lx], q2 = sm.pi[tp][1][ly][lx];
                    bool done = false;
                    if constexpr (FAST) {
                        const float psq = p1 * p1 + p2 * p2;
                        // float keeps 1/|psi|^4 finite only away from the cores' exact zeros
                        if (psq > 1e-15f && psq < 1e15f) {
                            float g[2][3];
                            const float wf = 0.0833333333f, wn = 0.666666667f;
#pragma unroll
                            for (int c = 0; c < 2; ++c) {
                                g[c][0] = (wf * (sm.ps[s0][c][hy][hx - 2] - sm.ps[s0][c][hy][hx + 2]) +
                                           wn * (sm.ps[s0][c][hy][hx + 1] - sm.ps[s0][c][hy][hx - 1])) * q.f_one_over_dx;
                                g[c][1] = (wf * (sm.ps[s0][c][hy - 2][hx] - sm.ps[s0][c][hy + 2][hx]) +
                                           wn * (sm.ps[s0][c][hy + 1][hx] - sm.ps[s0][c][hy - 1][hx])) * q.f_one_over_dx;
                                g[c][2] = (wf * (sm.ps[sm2][c][hy][hx] - sm.ps[sp2][c][hy][hx]) +
                                           wn * (sm.ps[sp1][c][hy][hx] - sm.ps[sm1][c][hy][hx])) * q.f_one_over_dx;
                            }
                            float term[6], wgt;
                            cell_energy<float, T>(kf, q.scheme, p1, p2, q1, q2, g, term, wgt);
#pragma unroll
                            for (int k = 0; k < 6; ++k) {
                                csum(ef[2 * k], ec[2 * k], term[k]);
                                csum(ef[2 * k + 1], ec[2 * k + 1], term[k] * wgt);
                            }
                            csum(ef[12], ec[12], wgt);
                            ef[13] += 1.f;
                            done = true;
                        }
                    }
                    if (!done) {
                        double g[2][3], term[6], wgt;
                        if constexpr (sizeof(T) == 4) {
                            // FP32 fields: taps widened by integer operations (f2d_exact)
                            float gf[2][3];
#pragma unroll
                            for (int c = 0; c < 2; ++c) {
                                g[c][0] = diff1_f32(sm.ps[s0][c][hy][hx - 2], sm.ps[s0][c][hy][hx - 1],
                                                    sm.ps[s0][c][hy][hx + 1], sm.ps[s0][c][hy][hx + 2], q.one_over_dx,
                                                    gf[c][0]);
                                g[c][1] = diff1_f32(sm.ps[s0][c][hy - 2][hx], sm.ps[s0][c][hy - 1][hx],
                                                    sm.ps[s0][c][hy + 1][hx], sm.ps[s0][c][hy + 2][hx], q.one_over_dx,
                                                    gf[c][1]);
                                g[c][2] = diff1_f32(sm.ps[sm2][c][hy][hx], sm.ps[sm1][c][hy][hx],
                                                    sm.ps[sp1][c][hy][hx], sm.ps[sp2][c][hy][hx], q.one_over_dx,
                                                    gf[c][2]);
                            }
                            cell_energy_g<double, float>(kd, q.scheme, f2d_exact(p1), f2d_exact(p2), f2d_exact(q1),
                                                         f2d_exact(q2), g, gf, term, wgt);
                        } else {
#pragma unroll
                            for (int c = 0; c < 2; ++c) {
                                g[c][0] = diff1_vals<T>(sm.ps[s0][c][hy][hx - 2], sm.ps[s0][c][hy][hx - 1],
                                                        sm.ps[s0][c][hy][hx + 1], sm.ps[s0][c][hy][hx + 2],
                                                        q.one_over_dx);
                                g[c][1] = diff1_vals<T>(sm.ps[s0][c][hy - 2][hx], sm.ps[s0][c][hy - 1][hx],
                                                        sm.ps[s0][c][hy + 1][hx], sm.ps[s0][c][hy + 2][hx],
                                                        q.one_over_dx);
                                g[c][2] = diff1_vals<T>(sm.ps[sm2][c][hy][hx], sm.ps[sm1][c][hy][hx],
                                                        sm.ps[sp1][c][hy][hx], sm.ps[sp2][c][hy][hx], q.one_over_dx);
                            }
                            cell_energy<double, T>(kd, q.scheme, p1, p2, q1, q2, g, term, wgt);
                        }
#pragma unroll
                        for (int k = 0; k < 6; ++k) {
                            e[2 * k] += term[k];
                            e[2 * k + 1] += term[k] * wgt;
                        }
                        e[12] += wgt;
                        e[13] += 1.0;
                    }
                }
                if (q.want_plaq || q.want_vel) {
                    // corner phases (x, y, z offsets) in the reference's order
                    const float f000 = sm.th[t0][ly][lx], f100 = sm.th[t0][ly][lx + 1];
                    const float f110 = sm.th[t0][ly + 1][lx + 1], f010 = sm.th[t0][ly + 1][lx];
                    const float f001 = sm.th[t1][ly][lx], f101 = sm.th[t1][ly][lx + 1], f011 = sm.th[t1][ly + 1][lx];
                    const bool ok = sm.ok[t0][ly][lx] & sm.ok[t0][ly][lx + 1] & sm.ok[t0][ly + 1][lx + 1] &
                                    sm.ok[t0][ly + 1][lx] & sm.ok[t1][ly][lx] & sm.ok[t1][ly][lx + 1] &
                                    sm.ok[t1][ly + 1][lx];
                    bool fast = ok;
                    if (fast) fast = winding4_fast(f000, f100, f110, f010, w[0]);
                    if (fast) fast = winding4_fast(f000, f010, f011, f001, w[1]);
                    if (fast) fast = winding4_fast(f000, f001, f101, f100, w[2]);
                    if (!fast) {
                        // near the branch cut or outside the float range: the reference's
                        // double arithmetic for this cell's three plaquettes
                        auto dph = [&](int slot, int ox_, int oy_) {
                            return atan2((double)sm.ps[slot][1][hy + oy_][hx + ox_],
                                         (double)sm.ps[slot][0][hy + oy_][hx + ox_]);
                        };
                        const double d000 = dph(s0, 0, 0), d100 = dph(s0, 1, 0), d110 = dph(s0, 1, 1);
                        const double d010 = dph(s0, 0, 1), d001 = dph(sp1, 0, 0), d101 = dph(sp1, 1, 0);
                        const double d011 = dph(sp1, 0, 1);
                        int ties = 0;
                        w[0] = winding4(d000, d100, d110, d010, ties);
                        w[1] = winding4(d000, d010, d011, d001, ties);
                        w[2] = winding4(d000, d001, d101, d100, ties);
                        cnt[3] += ties;
                    }
                    // StringTagger (StringTagger.hpp:117-151): a cell is tagged when a
                    // plaquette at its low corner is pierced
                    if (tags != nullptr) tags[cell] = (w[0] | w[1] | w[2]) != 0;
                    cnt[0] += (w[0] != 0) + (w[1] != 0) + (w[2] != 0);
                    cnt[1] += abs(w[0]) + abs(w[1]) + abs(w[2]);
                    if (q.want_vel && (w[0] | w[1] | w[2])) {
                        const double g000 = sm.gv[t0][ly][lx], g100 = sm.gv[t0][ly][lx + 1];
                        const double g110 = sm.gv[t0][ly + 1][lx + 1], g010 = sm.gv[t0][ly + 1][lx];
                        const double g001 = sm.gv[t1][ly][lx], g101 = sm.gv[t1][ly][lx + 1];
                        const double g011 = sm.gv[t1][ly + 1][lx];
                        double s = 0.0;
                        long long c = 0;
                        if (w[0]) { s += g000 + g100 + g110 + g010; c += 4; }
                        if (w[1]) { s += g000 + g010 + g011 + g001; c += 4; }
                        if (w[2]) { s += g000 + g001 + g101 + g100; c += 4; }
                        vsum += s;
                        cnt[2] += c;
                    }
                }
            }
            // ---- pierced plaquettes of this plane into the block's buffer: a warp
            // scan and one shared-memory atomic per warp that has any ----
            if (q.want_plaq && list != nullptr) {
                const int mine = (w[0] != 0) + (w[1] != 0) + (w[2] != 0);
                if (__any_sync(0xffffffffu, mine != 0)) {
                    const int lane = tid & 31;
                    int incl = mine;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int yv = __shfl_up_sync(0xffffffffu, incl, o);
                        if (lane >= o) incl += yv;
                    }
                    const int wtot = __shfl_sync(0xffffffffu, incl, 31);
                    int wbase = 0;
                    if (lane == 31) wbase = atomicAdd(&lcount, wtot);
                    wbase = __shfl_sync(0xffffffffu, wbase, 31);
                    warp_end = wbase + wtot;
                    int pos = wbase + incl - mine;
                    for (int pl = 0; pl < 3; ++pl)
                        if (w[pl]) sm.lbuf[pos++] = 4LL * cell + pl;
                }
            }
        }
        __syncthreads();  // the next item's prologue refills the rings
        if constexpr (FAST) {
#pragma unroll
            for (int k = 0; k < 14; ++k) {
                e[k] += (double)ef[k] + (k < 13 ? (double)ec[k < 13 ? k : 0] : 0.0);
                ef[k] = 0.f;
                if (k < 13) ec[k] = 0.f;
            }
        }
    }
    // the rest of the buffer (warp_end > 0: the warp appended since the last flush)
    if (q.want_plaq && list != nullptr && __syncthreads_or(warp_end > 0)) flush();

    // ---- block reduction (fixed order) ----
    __shared__ double red_d[kDiagThreads / 32][15];
    __shared__ long long red_l[kDiagThreads / 32][4];
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int s = 0; s < 14; ++s) {
        double xv = e[s];
        for (int o = 16; o > 0; o >>= 1) xv += __shfl_down_sync(0xffffffffu, xv, o);
        if (lane == 0) red_d[warp][s] = xv;
    }
    {
        double xv = vsum;
        for (int o = 16; o > 0; o >>= 1) xv += __shfl_down_sync(0xffffffffu, xv, o);
        if (lane == 0) red_d[warp][14] = xv;
    }
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        long long xv = cnt[s];
        for (int o = 16; o > 0; o >>= 1) xv += __shfl_down_sync(0xffffffffu, xv, o);
        if (lane == 0) red_l[warp][s] = xv;
    }
    __syncthreads();
    if (tid < 15) {
        double xv = 0.0;
        for (int ww = 0; ww < kDiagThreads / 32; ++ww) xv += red_d[ww][tid];
        if (tid < 14)
            partials[blockIdx.x].e[tid] = xv;
        else
            partials[blockIdx.x].vsum = xv;
    } else if (tid >= 32 && tid < 36) {
        long long xv = 0;
        for (int ww = 0; ww < kDiagThreads / 32; ++ww) xv += red_l[ww][tid - 32];
        partials[blockIdx.x].cnt[tid - 32] = xv;
    }
}

// ---------------------------------------------------------------- string finder
// The string finder and the tagger's plaquette criterion alone (no energy, no
// velocity). A block owns a FTX x FTY tile of cells, two cells per thread, and
// marches in z. Each fold decision is made once per edge: the winding of a
// plaquette is the signed sum of its four edges' folds, #(d < -pi) - #(d > pi)
// of the edge's phase difference d, and a plaquette walks an edge backwards
// with exactly -d, so it adds exactly minus the forward fold. That is the
// single-precision fast path of the fused pass edge for edge, with the same
// fall back to the reference's double arithmetic: a cell is redone in double
// when one of its nine edges lies within 1e-5 of +-pi or ends at a vertex
// outside float range. Those cells are queued in shared memory and redone
// after the z-chunk, outside the plane loop, so the rare double path costs
// the loop no registers; a chunk with more than the queue holds is searched
// again for them. Per vertex plane, with one block barrier:
//   B: the x and y edge codes of the plane before, from the neighbours' phases;
//   A: the thread's vertices' phases, from psi loaded into registers two
//      planes ahead, and their z edges to the plane below (phase kept in a
//      register);
//   C: the windings of the cells three planes back.
// Four slots per vertex-plane array keep every write two barriers from the
// last read of its slot.
constexpr int FTX = 32, FTY = 16, FVX = FTX + 1, FVY = FTY + 1;
constexpr int kFinderExtra = FTX + FTY + 1;  // vertices of the last row (x < FTX) and last column
constexpr int kFinderListBuf = 3072, kFinderFlushAt = kFinderListBuf - 6 * kDiagThreads;
constexpr int kFinderBadQ = 1024;  // cells queued for the double path per z-chunk
static_assert(FTX * FTY == 2 * kDiagThreads && kFinderExtra <= kDiagThreads, "two cells, at most three vertices per thread");

struct FinderSmem {
    long long lbuf[kFinderListBuf];
    int badq[kFinderBadQ];           // tile-local x | y << 5 | (z - za) << 9
    float th[4][FVY][FVX];           // phases of vertex plane p in slot p mod 4
    unsigned char ok[4][FVY][FVX];   // the vertex lies inside float range
    unsigned char inp[4][FVY][FVX];  // x edge code (bits 0-2), y edge code (bits 3-5)
    unsigned char zc[4][FVY][FVX];   // z edge code to the plane above (bits 0-2)
    float gv[4][FVY][FVX];           // gamma^2 v^2 of the vertex (velocity mode)
};

// gamma^2 v^2 at a vertex (Velocity.hpp:62-78 with the prefactors folded on the
// host) in single precision, with every operation rounded as written so that the
// plane pass and the after-chunk path agree to the bit
__device__ __forceinline__ float vertex_gv(float psi1, float psi2, float Pi1, float Pi2, const DiagConst &q)
{
    const float phi1 = __fmul_rn(psi1, q.f_inv_R), phi2 = __fmul_rn(psi2, q.f_inv_R);
    const float pd1 = __fmul_rn(__fsub_rn(Pi1, __fmul_rn(q.f_RpR, psi1)), q.f_inv_R2);
    const float pd2 = __fmul_rn(__fsub_rn(Pi2, __fmul_rn(q.f_RpR, psi2)), q.f_inv_R2);
    const float phi_sq = __fadd_rn(__fmul_rn(phi1, phi1), __fmul_rn(phi2, phi2));
    const float pd_sq = __fadd_rn(__fmul_rn(pd1, pd1), __fmul_rn(pd2, pd2));
    const float re = __fadd_rn(__fmul_rn(phi1, pd1), __fmul_rn(phi2, pd2));
    return __fsub_rn(__fmul_rn(__fmul_rn(pd_sq, q.f_vel_a), __fsub_rn(1.f, __fmul_rn(q.f_vel_b, phi_sq))),
                     __fmul_rn(__fmul_rn(q.f_vel_c, re), re));
}

struct CellWindings {
    int w[3], ties;
};

// edge code: fold + 1 in bits 0-1, bit 2 set when the cell must be redone in
// double (winding4_fast's band test on the same float difference)
__device__ __forceinline__ unsigned edge_code(float ta, float tb, bool ok)
{
    const float pi = 3.14159265f, band = 1e-5f;
    const float d = tb - ta;
    const bool bad = !ok || fabsf(fabsf(d) - pi) < band;
    return (unsigned)(1 + (d < -pi) - (d > pi)) | (bad ? 4u : 0u);
}
__device__ __forceinline__ int edge_fold(unsigned c) { return (int)(c & 3u) - 1; }

// A cell's three windings in the reference's double arithmetic, psi read from
// global memory at its seven corners (zero outside the view's ghost region, as
// the plane loads fill it). Out of line: it is rare and needs many registers.
template <typename T>
__device__ __noinline__ CellWindings finder_cell_double(const DiagView v, const T *base, int x, int y, int z)
{
    auto ph = [&](int xx, int yy, int zz) {
        const bool on = (v.wx || xx < v.nx + v.ox) && (v.wy || yy < v.ny + v.oy) && (v.wz || zz < v.nz + v.oz);
        const double a = on ? (double)base[view_off<T>(v, 0, xx, yy, zz)] : 0.0;
        const double b = on ? (double)base[view_off<T>(v, 1, xx, yy, zz)] : 0.0;
        return atan2(b, a);
    };
    const double d000 = ph(x, y, z), d100 = ph(x + 1, y, z), d110 = ph(x + 1, y + 1, z), d010 = ph(x, y + 1, z);
    const double d001 = ph(x, y, z + 1), d101 = ph(x + 1, y, z + 1), d011 = ph(x, y + 1, z + 1);
    CellWindings r;
    r.ties = 0;
    cell_windings_double(d000, d100, d110, d010, d001, d101, d011, r.w, r.ties);
    return r;
}

// Whether the finder sends a cell to the double path: one of its seven
// vertices outside float range, or one of its nine edges inside the band
// (edge_code's test on the same float phases).
template <typename T>
__device__ __noinline__ bool finder_cell_bad(const DiagView v, const T *base, int x, int y, int z)
{
    float th[8];
    bool ok[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int xx = x + (c & 1), yy = y + ((c >> 1) & 1), zz = z + (c >> 2);
        const bool on = (v.wx || xx < v.nx + v.ox) && (v.wy || yy < v.ny + v.oy) && (v.wz || zz < v.nz + v.oz);
        const T a = on ? base[view_off<T>(v, 0, xx, yy, zz)] : T(0);
        const T b = on ? base[view_off<T>(v, 1, xx, yy, zz)] : T(0);
        if constexpr (sizeof(T) == 4) {
            const float m = fmaxf(fabsf(a), fabsf(b));
            ok[c] = m > 1e-30f && m < 1e30f;
        } else {
            const double m = fmax(fabs(a), fabs(b));
            ok[c] = m > 1e-30 && m < 1e30;
        }
        th[c] = atan2f((float)b, (float)a);
    }
    // corners c = x + 2 y + 4 z; edges x: 0-1, 2-3, 4-5; y: 0-2, 1-3, 4-6; z: 0-4, 1-5, 2-6
    const int ea[9] = {0, 2, 4, 0, 1, 4, 0, 1, 2}, eb[9] = {1, 3, 5, 2, 3, 6, 4, 5, 6};
    unsigned bad = 0;
#pragma unroll
    for (int e = 0; e < 9; ++e) bad |= edge_code(th[ea[e]], th[eb[e]], ok[ea[e]] && ok[eb[e]]);
    return (bad & 4u) != 0;
}

// VEL (FP32 fields, beside energy32_kernel): also Pi at the vertices, gamma^2 v^2
// per vertex and its sum over the corners of every pierced plaquette. Blocks from
// e_from on clear their partial record's energy sums (energy32_kernel writes those
// of the blocks below it).
template <typename T, bool VEL>
__global__ void __launch_bounds__(kDiagThreads, (sizeof(T) == 4 && !VEL) ? 4 : 3)
    finder_kernel(const DiagView v, const DiagConst q, const uint8_t *__restrict__ mask,
                  DiagPartial *__restrict__ partials, unsigned long long *__restrict__ list_counter,
                  long long *__restrict__ list, long long capacity, int tiles_x, int ntiles, int zchunk,
                  long long n_items, long long items_per_box, int64_t box_stride, uint8_t *__restrict__ tags,
                  int e_from)
{
    extern __shared__ __align__(16) unsigned char finder_smem_raw[];
    FinderSmem &sm = *reinterpret_cast<FinderSmem *>(finder_smem_raw);
    __shared__ int lcount, flush_n, badn, bad_over;
    __shared__ unsigned long long flush_base;
    __shared__ long long red[kDiagThreads / 32][4];
    const int tid = threadIdx.x, lane = tid & 31;
    const int lx = tid % FTX, ly = tid / FTX;  // cells (lx, ly) and (lx, ly + FTY / 2)
    const int64_t box_cells = (int64_t)v.nx * v.ny * v.nz;
    int cnt_p = 0, cnt_w = 0, cnt_tie = 0;  // per-thread counts fit 32 bits
    // velocity mode: corner sums in FP32, a chunk's running sum compensated (Neumaier),
    // FP64 across chunks (GB300 issues FP64 at 1/64 of the FP32 rate)
    int cnt_v = 0;
    double vsum = 0.0;
    float vacc = 0.f, vcomp = 0.f;
    auto vadd = [&](float x) {
        const float t = vacc + x;
        vcomp += fabsf(vacc) >= fabsf(x) ? (vacc - t) + x : (x - t) + vacc;
        vacc = t;
    };
    if (tid == 0) lcount = badn = bad_over = 0;
    int warp_end = 0;  // end of this warp's last append to lbuf (lane-uniform)
    auto flush = [&]() {
        if (tid == 0) {
            const int nb = lcount;
            flush_n = nb;
            flush_base = nb ? atomicAdd(list_counter, (unsigned long long)nb) : 0ull;
            lcount = 0;
        }
        __syncthreads();
        const int nb = flush_n;
        const unsigned long long b0 = flush_base;
        for (int i = tid; i < nb; i += kDiagThreads)
            if (b0 + i < (unsigned long long)capacity) list[b0 + i] = sm.lbuf[i];
        __syncthreads();
        warp_end = 0;
    };
    // a cell of the double path: windings, counts, tag and list entries (one
    // global atomic each: these cells are rare)
    auto redo_cell = [&](const T *base, long long qbox, int x, int y, int z) {
        const CellWindings cw = finder_cell_double<T>(v, base, x, y, z);
        const int64_t cell = qbox * box_cells + (int64_t)x + (int64_t)v.nx * ((int64_t)y + (int64_t)v.ny * z);
        cnt_tie += cw.ties;
        if (tags != nullptr) tags[cell] = (cw.w[0] | cw.w[1] | cw.w[2]) != 0;
        if constexpr (VEL) {
            if (cw.w[0] | cw.w[1] | cw.w[2]) {
                // gamma^2 v^2 at the corners, from global memory (zero outside the ghost region)
                auto gvat = [&](int dx_, int dy_, int dz_) -> float {
                    const int xx = x + dx_, yy = y + dy_, zz = z + dz_;
                    const bool on =
                        (v.wx || xx < v.nx + v.ox) && (v.wy || yy < v.ny + v.oy) && (v.wz || zz < v.nz + v.oz);
                    float c4[4];
                    for (int c = 0; c < 4; ++c) c4[c] = on ? (float)base[view_off<T>(v, c, xx, yy, zz)] : 0.f;
                    return vertex_gv(c4[0], c4[1], c4[2], c4[3], q);
                };
                const float g000 = gvat(0, 0, 0), g100 = gvat(1, 0, 0), g110 = gvat(1, 1, 0), g010 = gvat(0, 1, 0);
                const float g001 = gvat(0, 0, 1), g101 = gvat(1, 0, 1), g011 = gvat(0, 1, 1);
                float s_ = 0.f;
                if (cw.w[0]) { s_ += g000 + g100 + g110 + g010; cnt_v += 4; }
                if (cw.w[1]) { s_ += g000 + g010 + g011 + g001; cnt_v += 4; }
                if (cw.w[2]) { s_ += g000 + g001 + g101 + g100; cnt_v += 4; }
                vadd(s_);
            }
        }
#pragma unroll
        for (int pl = 0; pl < 3; ++pl) {
            if (!cw.w[pl]) continue;
            ++cnt_p;
            cnt_w += abs(cw.w[pl]);
            if (list != nullptr) {
                const unsigned long long pos = atomicAdd(list_counter, 1ull);
                if (pos < (unsigned long long)capacity) list[pos] = 4LL * cell + pl;
            }
        }
    };

    // the thread's vertices: (lx, ly), (lx, ly + 8) and, for the first 49
    // threads, one of the last row (y = FTY) or the last column (x = FTX)
    const bool extra = tid < kFinderExtra;
    const int vi[3] = {lx, lx, tid < FTX ? tid : FTX};
    const int vj[3] = {ly, ly + FTY / 2, tid < FTX ? FTY : (extra ? tid - FTX : 0)};

    for (long long item = blockIdx.x; item < n_items; item += gridDim.x) {
        const long long qbox = item / items_per_box, box_item = item % items_per_box;
        const T *__restrict__ base = static_cast<const T *>(v.data) + qbox * box_stride;
        const int tile = (int)(box_item % ntiles), chunk = (int)(box_item / ntiles);
        const int x0 = (tile % tiles_x) * FTX, y0 = (tile / tiles_x) * FTY;
        const int za = chunk * zchunk, len = min(zchunk, v.nz - za);

        // in-plane element offsets of the thread's vertices (the host checks that
        // a plane's offsets fit 31 bits), -1 outside the ghost region: psi is zero there
        int voff[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int xx = x0 + vi[k], yy = y0 + vj[k];
            const bool on = (k < 2 || extra) && xx <= v.nx && yy <= v.ny && (v.wx || xx < v.nx + v.ox) &&
                            (v.wy || yy < v.ny + v.oy);
            voff[k] = on ? (wrap_or_self(xx, v.nx, v.wx) + v.ox) + (wrap_or_self(yy, v.ny, v.wy) + v.oy) * (int)v.js
                         : -1;
        }
        // psi of vertex planes za, za + 1, ... in order, into registers
        int lz = za, lzw = wrap_or_self(za, v.nz, v.wz);
        constexpr int NC = VEL ? 4 : 2;  // psi (and Pi) at the vertices
        auto load_plane = [&](T(&buf)[3][NC]) {
            const bool zin = v.wz || lz < v.nz + v.oz;
            const T *pb = base + (int64_t)(lzw + v.oz) * v.ks;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const bool on = zin && voff[k] >= 0;
#pragma unroll
                for (int c = 0; c < NC; ++c) buf[k][c] = on ? __ldg(pb + voff[k] + c * v.cs) : T(0);
            }
            ++lz;
            lzw = v.wz ? (lzw + 1 == v.nz ? 0 : lzw + 1) : lzw + 1;
        };
        float thp[3];  // phase and range flag of the vertex one plane down
        bool okp[3];

        // B: x and y edge codes of vertex plane za + j - 1
        auto stage_b = [&](int j) {
            const int s = (j - 1) & 3;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (k == 2 && !extra) break;
                const int i = vi[k], jj = vj[k];
                unsigned code = 0;
                if (i < FTX) code = edge_code(thp[k], sm.th[s][jj][i + 1], okp[k] && sm.ok[s][jj][i + 1]);
                if (jj < FTY) code |= edge_code(thp[k], sm.th[s][jj + 1][i], okp[k] && sm.ok[s][jj + 1][i]) << 3;
                sm.inp[s][jj][i] = (unsigned char)code;
            }
        };
        // A: phases of vertex plane za + j and the z edges from plane za + j - 1
        auto stage_a = [&](int j, const T(&buf)[3][NC]) {
            const int s = j & 3, sp = (j - 1) & 3;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (k == 2 && !extra) break;
                const T a = buf[k][0], b = buf[k][1];
                bool ok;
                if constexpr (sizeof(T) == 4) {
                    const float m = fmaxf(fabsf(a), fabsf(b));
                    ok = m > 1e-30f && m < 1e30f;
                } else {
                    const double m = fmax(fabs(a), fabs(b));
                    ok = m > 1e-30 && m < 1e30;
                }
                const float th = atan2f((float)b, (float)a);
                sm.th[s][vj[k]][vi[k]] = th;
                sm.ok[s][vj[k]][vi[k]] = ok;
                if constexpr (VEL) sm.gv[s][vj[k]][vi[k]] = vertex_gv((float)a, (float)b, (float)buf[k][2], (float)buf[k][3], q);
                if (j > 0) sm.zc[sp][vj[k]][vi[k]] = (unsigned char)edge_code(thp[k], th, okp[k] && ok);
                thp[k] = th;
                okp[k] = ok;
            }
        };
        // C: windings of the cells of plane za + j - 3
        auto stage_c = [&](int j) {
            const int s0 = (j - 3) & 3, s1 = (j - 2) & 3, z = za + j - 3;
            // cell index of (lx, ly) and the step to (lx, ly + FTY / 2)
            const int64_t cell0 = qbox * box_cells + (int64_t)(x0 + lx) +
                                  (int64_t)v.nx * ((int64_t)(y0 + ly) + (int64_t)v.ny * z);
            const int64_t hstep = (int64_t)v.nx * (FTY / 2);
            unsigned pm = 0;  // pierced plaquettes: bit 3 h + plane
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int cy = ly + h * (FTY / 2), x = x0 + lx, y = y0 + cy;
                if (!(x < v.nx && y < v.ny)) continue;
                const int64_t cell = cell0 + h * hstep;
                if (mask != nullptr && mask[cell] == 0) continue;
                const unsigned c000 = sm.inp[s0][cy][lx], c100 = sm.inp[s0][cy][lx + 1];
                const unsigned c010 = sm.inp[s0][cy + 1][lx], c001 = sm.inp[s1][cy][lx];
                const unsigned z000 = sm.zc[s0][cy][lx], z100 = sm.zc[s0][cy][lx + 1], z010 = sm.zc[s0][cy + 1][lx];
                const unsigned bad =
                    ((c000 | c001) & 0x24u) | (c100 & 0x20u) | (c010 & 0x04u) | ((z000 | z100 | z010) & 0x04u);
                if (bad) {
                    // the double path after the chunk
                    const int slot = atomicAdd(&badn, 1);
                    if (slot < kFinderBadQ)
                        sm.badq[slot] = lx | (cy << 5) | ((z - za) << 9);
                    else
                        bad_over = 1;
                    continue;
                }
                // StringFinder.hpp:45-68 order: xy (000 100 110 010), yz (000 010 011 001), zx (000 001 101 100)
                const int wxy = edge_fold(c000) + edge_fold(c100 >> 3) - edge_fold(c010) - edge_fold(c000 >> 3);
                const int wyz = edge_fold(c000 >> 3) + edge_fold(z010) - edge_fold(c001 >> 3) - edge_fold(z000);
                const int wzx = edge_fold(z000) + edge_fold(c001) - edge_fold(z100) - edge_fold(c000);
                const unsigned cm = (wxy != 0) | (wyz != 0) << 1 | (wzx != 0) << 2;
                // StringTagger.hpp:117-151: a cell is tagged when a plaquette at its low corner is pierced
                if (tags != nullptr) tags[cell] = cm != 0;
                if constexpr (VEL) {
                    // VelocityKernel.hpp:37-141: gamma^2 v^2 of the 4 corners of every pierced plaquette
                    if (cm) {
                        const float g000 = sm.gv[s0][cy][lx], g100 = sm.gv[s0][cy][lx + 1];
                        const float g110 = sm.gv[s0][cy + 1][lx + 1], g010 = sm.gv[s0][cy + 1][lx];
                        const float g001 = sm.gv[s1][cy][lx], g101 = sm.gv[s1][cy][lx + 1];
                        const float g011 = sm.gv[s1][cy + 1][lx];
                        float s_ = 0.f;
                        if (wxy) { s_ += g000 + g100 + g110 + g010; cnt_v += 4; }
                        if (wyz) { s_ += g000 + g010 + g011 + g001; cnt_v += 4; }
                        if (wzx) { s_ += g000 + g001 + g101 + g100; cnt_v += 4; }
                        vadd(s_);
                    }
                }
                cnt_w += abs(wxy) + abs(wyz) + abs(wzx);
                pm |= cm << (3 * h);
            }
            const int mine = __popc(pm);
            cnt_p += mine;
            // pierced plaquettes into the block's buffer: a warp scan and one
            // shared-memory atomic per warp that has any
            if (list != nullptr && __any_sync(0xffffffffu, mine != 0)) {
                int incl = mine;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int yv = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += yv;
                }
                const int wtot = __shfl_sync(0xffffffffu, incl, 31);
                int wbase = 0;
                if (lane == 31) wbase = atomicAdd(&lcount, wtot);
                wbase = __shfl_sync(0xffffffffu, wbase, 31);
                warp_end = wbase + wtot;
                int pos = wbase + incl - mine;
                const long long e0 = 4LL * cell0, eh = 4LL * hstep - 3;
                while (pm) {
                    const int b = __ffs(pm) - 1;
                    pm &= pm - 1;
                    sm.lbuf[pos++] = e0 + b + (b >= 3 ? eh : 0);  // 4 cell + plane
                }
            }
        };
        // iteration j: B (plane za + j - 1), A (plane za + j, then the load of
        // plane za + j + 2 into the registers A just read), C (cells of plane
        // za + j - 3); the loop is unrolled by two so each register buffer has
        // a fixed name
        auto step = [&](int j, T(&buf)[3][NC]) {
            // the plane's one barrier; the block also learns whether the pierced
            // buffer could overflow during this plane
            if (__syncthreads_or(warp_end > kFinderFlushAt)) flush();
            if (j >= 1 && j <= len + 1) stage_b(j);
            if (j <= len) {
                stage_a(j, buf);
                if (j + 2 <= len) load_plane(buf);
            }
            if (j >= 3) stage_c(j);
        };
        T bufa[3][NC], bufb[3][NC];
        load_plane(bufa);  // vertex plane za
        load_plane(bufb);  // za + 1 (len >= 1)
        for (int j = 0; j < len + 3; j += 2) {
            step(j, bufa);
            if (j + 1 < len + 3) step(j + 1, bufb);
        }
        // the chunk's double-path cells: from the queue, or, when it overflowed,
        // by testing every cell of the chunk again
        __syncthreads();
        const int nbad = badn;
        if (!bad_over) {
            for (int i = tid; i < nbad; i += kDiagThreads) {
                const int e = sm.badq[i];
                redo_cell(base, qbox, x0 + (e & 31), y0 + ((e >> 5) & 15), za + (e >> 9));
            }
        } else {
            for (int c = tid; c < FTX * FTY * len; c += kDiagThreads) {
                const int x = x0 + c % FTX, y = y0 + (c / FTX) % FTY, z = za + c / (FTX * FTY);
                if (x >= v.nx || y >= v.ny) continue;
                if (mask != nullptr &&
                    mask[qbox * box_cells + x + (int64_t)v.nx * ((int64_t)y + (int64_t)v.ny * z)] == 0)
                    continue;
                if (finder_cell_bad<T>(v, base, x, y, z)) redo_cell(base, qbox, x, y, z);
            }
        }
        __syncthreads();
        if (tid == 0) badn = bad_over = 0;  // published by the next chunk's first barrier
        if constexpr (VEL) {
            vsum += (double)vacc + (double)vcomp;
            vacc = vcomp = 0.f;
        }
    }
    if (list != nullptr && __syncthreads_or(warp_end > 0)) flush();

    // ---- block reduction (fixed order) into the fused pass's partial record ----
    __shared__ double redv[kDiagThreads / 32];
    long long c4[4] = {cnt_p, cnt_w, VEL ? cnt_v : 0, cnt_tie};
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        for (int o = 16; o > 0; o >>= 1) c4[s] += __shfl_down_sync(0xffffffffu, c4[s], o);
        if (lane == 0) red[tid >> 5][s] = c4[s];
    }
    if constexpr (VEL)
        for (int o = 16; o > 0; o >>= 1) vsum += __shfl_down_sync(0xffffffffu, vsum, o);
    if (lane == 0) redv[tid >> 5] = VEL ? vsum : 0.0;
    __syncthreads();
    if (tid < 14) {
        if ((int)blockIdx.x >= e_from) partials[blockIdx.x].e[tid] = 0.0;
    } else if (tid == 14) {
        double xv = 0.0;
        for (int ww = 0; ww < kDiagThreads / 32; ++ww) xv += redv[ww];
        partials[blockIdx.x].vsum = xv;
    } else if (tid >= 32 && tid < 36) {
        const int f = tid - 32;  // n_p_plain, n_p_weighted, vel_count, near_tie
        long long xv = 0;
        for (int ww = 0; ww < kDiagThreads / 32; ++ww) xv += red[ww][f];
        partials[blockIdx.x].cnt[f] = xv;
    }
}

// ---------------------------------------------------------------- FP32 per-cell energy sums
// The per_cell_fp32 energy sums on FP32 fields, run beside finder_kernel<float, VEL>
// (windings, the pierced list and the velocity), each kernel with few registers.
// A block owns a FTX x FTY tile, two cells per thread, and marches in z. psi of the
// tile plus a 2-cell halo arrives by cp.async in a ring of seven planes (the
// gradient stencil's five plus two, so one block barrier per plane suffices), Pi
// of the tile in a ring of three. Per plane each warp adds up its cells' 13 terms
// in FP32 with a butterfly over the lanes, and lane k adds sum k to a compensated
// (Neumaier) FP32 accumulator, lane 13 the cell count. After each z-chunk the
// accumulators go to per-warp FP64 slots. Cells where FP32 cannot hold 1/|psi|^4
// (|psi|^2 outside (1e-15, 1e15): the cores' exact zeros) are queued and take the
// reference's double arithmetic after the chunk, as the fused pass does.
constexpr int EHX = FTX + 4, EHY = FTY + 4, kEnergySlots = 7, kEnergyPiSlots = 3, kEnergyBadQ = 1024;
constexpr int kEnergyPts = 2 * EHX * EHY, kEnergyPer = (kEnergyPts + kDiagThreads - 1) / kDiagThreads;
constexpr int kEnergyPiPts = 2 * FTX * FTY, kEnergyPiPer = kEnergyPiPts / kDiagThreads;
static_assert(kEnergyPiPts % kDiagThreads == 0, "Pi loads per thread");
struct EnergySmem {
    double ew[kDiagThreads / 32][14];
    float ps[kEnergySlots][2][EHY][EHX];
    float pi[kEnergyPiSlots][2][FTY][FTX];
    int badq[kEnergyBadQ];  // tile-local x | y << 5 | (z - za) << 9
};

struct CellTerms {
    double t[14];
};

// One cell's 14 terms in the reference's double per-cell arithmetic, psi and Pi
// read from global memory (zero outside the view's ghost region).
__device__ __noinline__ CellTerms energy_cell_double(const DiagView v, const DiagConst q, const float *base, int x,
                                                     int y, int z)
{
    auto at = [&](int c, int xx, int yy, int zz) -> double {
        const bool on = (v.wx || (xx >= -v.ox && xx < v.nx + v.ox)) && (v.wy || (yy >= -v.oy && yy < v.ny + v.oy)) &&
                        (v.wz || (zz >= -v.oz && zz < v.nz + v.oz));
        return on ? (double)base[view_off<float>(v, c, xx, yy, zz)] : 0.0;
    };
    double g[2][3];
    for (int c = 0; c < 2; ++c) {
        g[c][0] = diff1_vals<float>(at(c, x - 2, y, z), at(c, x - 1, y, z), at(c, x + 1, y, z), at(c, x + 2, y, z),
                                    q.one_over_dx);
        g[c][1] = diff1_vals<float>(at(c, x, y - 2, z), at(c, x, y - 1, z), at(c, x, y + 1, z), at(c, x, y + 2, z),
                                    q.one_over_dx);
        g[c][2] = diff1_vals<float>(at(c, x, y, z - 2), at(c, x, y, z - 1), at(c, x, y, z + 1), at(c, x, y, z + 2),
                                    q.one_over_dx);
    }
    const CellConst<double> kd{q.R2, q.inv_R, q.inv_R2, q.inv_R4, q.lambda, q.RpR, q.threshold};
    double term[6], wgt;
    cell_energy<double, float>(kd, q.scheme, at(0, x, y, z), at(1, x, y, z), at(2, x, y, z), at(3, x, y, z), g, term,
                               wgt);
    CellTerms r;
    for (int k = 0; k < 6; ++k) {
        r.t[2 * k] = term[k];
        r.t[2 * k + 1] = term[k] * wgt;
    }
    r.t[12] = wgt;
    r.t[13] = 1.0;
    return r;
}

__global__ void __launch_bounds__(kDiagThreads, 3)
    energy32_kernel(const DiagView v, const DiagConst q, const uint8_t *__restrict__ mask,
                    DiagPartial *__restrict__ partials, int tiles_x, int ntiles, int zchunk, long long n_items,
                    long long items_per_box, int64_t box_stride, int zero_counts)
{
    extern __shared__ __align__(16) unsigned char energy_smem_raw[];
    EnergySmem &sm = *reinterpret_cast<EnergySmem *>(energy_smem_raw);
    __shared__ int badn, bad_over;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int lx = tid % FTX, ly = tid / FTX;  // cells (lx, ly) and (lx, ly + FTY / 2)
    const int64_t box_cells = (int64_t)v.nx * v.ny * v.nz;
    const CellConst<float> kf{q.f_R2, q.f_inv_R, q.f_inv_R2, q.f_inv_R4, q.f_lambda, q.f_RpR, q.f_threshold};
    for (int i = tid; i < (kDiagThreads / 32) * 14; i += kDiagThreads) sm.ew[i / 14][i % 14] = 0.0;
    if (tid == 0) badn = bad_over = 0;
    float acc = 0.f, comp = 0.f;  // lane k < 13: running sum k of the chunk; lane 13: its cell count

    for (long long item = blockIdx.x; item < n_items; item += gridDim.x) {
        const long long qbox = item / items_per_box, box_item = item % items_per_box;
        const float *__restrict__ base = static_cast<const float *>(v.data) + qbox * box_stride;
        const int tile = (int)(box_item % ntiles), chunk = (int)(box_item / ntiles);
        const int x0 = (tile % tiles_x) * FTX, y0 = (tile / tiles_x) * FTY;
        const int za = chunk * zchunk, len = min(zchunk, v.nz - za);

        // load plans (in-plane offsets in 31 bits, checked on the host; -1: zero fill)
        int poff[kEnergyPer];
#pragma unroll
        for (int u = 0; u < kEnergyPer; ++u) {
            const int idx = tid + u * kDiagThreads, r = idx % (EHX * EHY);
            const int xx = x0 - 2 + r % EHX, yy = y0 - 2 + r / EHX;
            const bool on = idx < kEnergyPts && xx < v.nx + 2 && yy < v.ny + 2 &&
                            (v.wx || (xx >= -v.ox && xx < v.nx + v.ox)) && (v.wy || (yy >= -v.oy && yy < v.ny + v.oy));
            poff[u] = on ? (wrap_or_self(xx, v.nx, v.wx) + v.ox) + (wrap_or_self(yy, v.ny, v.wy) + v.oy) * (int)v.js
                         : -1;
        }
        int qoff[kEnergyPiPer];
#pragma unroll
        for (int u = 0; u < kEnergyPiPer; ++u) {
            const int idx = tid + u * kDiagThreads, r = idx % (FTX * FTY);
            const int xx = x0 + r % FTX, yy = y0 + r / FTX;
            qoff[u] = xx < v.nx && yy < v.ny ? (xx + v.ox) + (yy + v.oy) * (int)v.js : -1;
        }
        // psi planes za - 2 .. za + len + 1 (plane p in slot (p - za + 2) mod 7), Pi planes
        // za .. za + len - 1 (slot (p - za) mod 3), each loaded in order
        int lz = za - 2, lzw = wrap_or_self(za - 2, v.nz, v.wz);
        auto load_psi_next = [&]() {
            const bool zin = v.wz || (lz >= -v.oz && lz < v.nz + v.oz);
            const float *pb = base + (int64_t)(lzw + v.oz) * v.ks;
            float *dst = &sm.ps[(lz - za + 2) % kEnergySlots][0][0][0];
#pragma unroll
            for (int u = 0; u < kEnergyPer; ++u) {
                const int idx = tid + u * kDiagThreads;
                if (idx < kEnergyPts)
                    cp_async_elem(dst + idx, pb + (idx >= EHX * EHY ? v.cs : 0) + poff[u], zin && poff[u] >= 0, base);
            }
            ++lz;
            lzw = v.wz ? (lzw + 1 == v.nz ? 0 : lzw + 1) : lzw + 1;
        };
        int pz = za, pzw = wrap_or_self(za, v.nz, v.wz);
        auto load_pi_next = [&]() {
            const float *pb = base + (int64_t)(pzw + v.oz) * v.ks + 2 * v.cs;
            float *dst = &sm.pi[(pz - za) % kEnergyPiSlots][0][0][0];
#pragma unroll
            for (int u = 0; u < kEnergyPiPer; ++u) {
                const int idx = tid + u * kDiagThreads;
                cp_async_elem(dst + idx, pb + (idx >= FTX * FTY ? v.cs : 0) + qoff[u], qoff[u] >= 0, base);
            }
            ++pz;
            pzw = v.wz ? (pzw + 1 == v.nz ? 0 : pzw + 1) : pzw + 1;
        };
        for (int p = 0; p < 5; ++p) load_psi_next();  // za - 2 .. za + 2
        load_pi_next();                               // za
        cp_async_commit();

        for (int m = 0; m < len; ++m) {
            const int z = za + m;
            // one plane ahead: psi(z + 3), Pi(z + 1); their slots were last read two planes back
            if (m + 1 < len) {
                load_psi_next();
                load_pi_next();
            }
            cp_async_commit();
            cp_async_wait<1>();  // psi(z + 2), Pi(z)
            __syncthreads();
            const int s0 = (m + 2) % kEnergySlots, sm1 = (m + 1) % kEnergySlots, sp1 = (m + 3) % kEnergySlots,
                      sm2 = m % kEnergySlots, sp2 = (m + 4) % kEnergySlots, tp = m % kEnergyPiSlots;
            float ts[13];
#pragma unroll
            for (int k = 0; k < 13; ++k) ts[k] = 0.f;
            int ncell = 0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int cy = ly + h * (FTY / 2), x = x0 + lx, y = y0 + cy;
                if (!(x < v.nx && y < v.ny)) continue;
                if (mask != nullptr &&
                    mask[qbox * box_cells + (int64_t)x + (int64_t)v.nx * ((int64_t)y + (int64_t)v.ny * z)] == 0)
                    continue;
                const int hx = lx + 2, hy = cy + 2;
                const float p1 = sm.ps[s0][0][hy][hx], p2 = sm.ps[s0][1][hy][hx];
                const float psq = p1 * p1 + p2 * p2;
                if (!(psq > 1e-15f && psq < 1e15f)) {
                    // the double path after the chunk
                    const int slot = atomicAdd(&badn, 1);
                    if (slot < kEnergyBadQ)
                        sm.badq[slot] = lx | (cy << 5) | ((z - za) << 9);
                    else
                        bad_over = 1;
                    continue;
                }
                float g[2][3];
                const float wf = 0.0833333333f, wn = 0.666666667f;
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    g[c][0] = (wf * (sm.ps[s0][c][hy][hx - 2] - sm.ps[s0][c][hy][hx + 2]) +
                               wn * (sm.ps[s0][c][hy][hx + 1] - sm.ps[s0][c][hy][hx - 1])) * q.f_one_over_dx;
                    g[c][1] = (wf * (sm.ps[s0][c][hy - 2][hx] - sm.ps[s0][c][hy + 2][hx]) +
                               wn * (sm.ps[s0][c][hy + 1][hx] - sm.ps[s0][c][hy - 1][hx])) * q.f_one_over_dx;
                    g[c][2] = (wf * (sm.ps[sm2][c][hy][hx] - sm.ps[sp2][c][hy][hx]) +
                               wn * (sm.ps[sp1][c][hy][hx] - sm.ps[sm1][c][hy][hx])) * q.f_one_over_dx;
                }
                float term[6], wgt;
                cell_energy<float, float>(kf, q.scheme, p1, p2, sm.pi[tp][0][cy][lx], sm.pi[tp][1][cy][lx], g,
                                          term, wgt);
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    ts[2 * k] += term[k];
                    ts[2 * k + 1] += term[k] * wgt;
                }
                ts[12] += wgt;
                ++ncell;
            }
            // the warp's sums of this plane (butterfly), then lane k's compensated accumulator
#pragma unroll
            for (int k = 0; k < 13; ++k)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) ts[k] += __shfl_xor_sync(0xffffffffu, ts[k], o);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ncell += __shfl_xor_sync(0xffffffffu, ncell, o);
            float mine = (float)ncell;
#pragma unroll
            for (int k = 0; k < 13; ++k)
                if (lane == k) mine = ts[k];
            if (lane < 13) {
                const float t = acc + mine;
                comp += fabsf(acc) >= fabsf(mine) ? (acc - t) + mine : (mine - t) + acc;
                acc = t;
            } else if (lane == 13) {
                acc += mine;  // cell counts stay exact in float: at most 512 per plane, 2^24 per chunk
            }
        }
        __syncthreads();  // the queue is complete; the rings are free for the next chunk
        if (lane < 14) sm.ew[warp][lane] += (double)acc + (double)comp;
        acc = comp = 0.f;
        // the chunk's double-path cells: from the queue or, when it overflowed, by testing
        // every cell again; each warp sums its cells' terms and lane k adds sum k
        const int nbad = badn;
        if (nbad > 0) {
            double d[14];
#pragma unroll
            for (int k = 0; k < 14; ++k) d[k] = 0.0;
            auto add_cell = [&](int x, int y, int z) {
                const CellTerms ct = energy_cell_double(v, q, base, x, y, z);
#pragma unroll
                for (int k = 0; k < 14; ++k) d[k] += ct.t[k];
            };
            if (!bad_over) {
                for (int i = tid; i < nbad; i += kDiagThreads) {
                    const int e = sm.badq[i];
                    add_cell(x0 + (e & 31), y0 + ((e >> 5) & 15), za + (e >> 9));
                }
            } else {
                for (int c = tid; c < FTX * FTY * len; c += kDiagThreads) {
                    const int x = x0 + c % FTX, y = y0 + (c / FTX) % FTY, z = za + c / (FTX * FTY);
                    if (x >= v.nx || y >= v.ny) continue;
                    if (mask != nullptr &&
                        mask[qbox * box_cells + x + (int64_t)v.nx * ((int64_t)y + (int64_t)v.ny * z)] == 0)
                        continue;
                    const float *pc = base + view_off<float>(v, 0, x, y, z);
                    const float p1 = pc[0], p2 = pc[v.cs], psq = p1 * p1 + p2 * p2;
                    if (!(psq > 1e-15f && psq < 1e15f)) add_cell(x, y, z);
                }
            }
#pragma unroll
            for (int k = 0; k < 14; ++k)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) d[k] += __shfl_xor_sync(0xffffffffu, d[k], o);
            double dm = 0.0;
#pragma unroll
            for (int k = 0; k < 14; ++k)
                if (lane == k) dm = d[k];
            if (lane < 14) sm.ew[warp][lane] += dm;
        }
        __syncthreads();
        if (tid == 0) badn = bad_over = 0;  // published by the next chunk's first barrier
    }
    __syncthreads();
    if (tid < 14) {
        double xv = 0.0;
        for (int ww = 0; ww < kDiagThreads / 32; ++ww) xv += sm.ew[ww][tid];
        partials[blockIdx.x].e[tid] = xv;
    } else if (zero_counts && tid == 14) {
        partials[blockIdx.x].vsum = 0.0;
    } else if (zero_counts && tid >= 32 && tid < 36) {
        partials[blockIdx.x].cnt[tid - 32] = 0;
    }
}

// Sum the per-block partials in a fixed pairwise order and write the result.
__global__ void diag_finalize_kernel(const DiagPartial *__restrict__ partials, int nblocks,
                                     const unsigned long long *__restrict__ list_counter, long long capacity,
                                     int want_list, axs_diag_result *__restrict__ out)
{
    __shared__ double sd[256];
    __shared__ long long sl[256];
    const int t = threadIdx.x;
    for (int f = 0; f < 19; ++f) {
        double xd = 0.0;
        long long xl = 0;
        for (int b = t; b < nblocks; b += 256) {
            if (f < 14)
                xd += partials[b].e[f];
            else if (f == 14)
                xd += partials[b].vsum;
            else
                xl += partials[b].cnt[f - 15];
        }
        sd[t] = xd;
        sl[t] = xl;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (t < o) {
                sd[t] += sd[t + o];
                sl[t] += sl[t + o];
            }
            __syncthreads();
        }
        if (t == 0) {
            if (f < 14)
                out->energy_sums[f] = sd[0];
            else if (f == 14)
                out->vel_sum = sd[0];
            else if (f == 15)
                out->n_p_plain = sl[0];
            else if (f == 16)
                out->n_p_weighted = sl[0];
            else if (f == 17)
                out->vel_count = sl[0];
            else
                out->n_near_tie = sl[0];
        }
        __syncthreads();
    }
    if (t == 0) {
        const long long listed = want_list ? (long long)*list_counter : 0;
        out->n_listed = listed < capacity ? listed : capacity;
        out->status = (want_list && listed > capacity) ? AXS_ERR_CAPACITY : AXS_OK;
    }
}

// Upper bound on the blocks a pass launches (the scratch is sized for it).
static int diag_grid(int64_t ncell)
{
    const int sms = device_sm_count();
    int64_t g = (ncell + kDiagThreads - 1) / kDiagThreads;
    const int64_t cap = (int64_t)(sms > 0 ? sms : 148) * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

// Work items (tile, z-chunk), tile fastest; chunks long enough to amortise
// the 4 warm-up planes while giving every resident block several items.
static void diag_plan(const DiagView &v, int nboxes, int max_grid, int tx, int ty, int blocks_per_sm, int &tiles_x,
                      int &ntiles, int &zchunk, long long &items_per_box, long long &items, int &grid)
{
    tiles_x = (v.nx + tx - 1) / tx;
    ntiles = tiles_x * ((v.ny + ty - 1) / ty);
    const int sms = device_sm_count() > 0 ? device_sm_count() : 148;
    const long long resident = (long long)blocks_per_sm * sms;
    const long long tiles_all = (long long)ntiles * nboxes;
    int nch = (int)std::max<long long>(1, (4 * resident + tiles_all - 1) / tiles_all);
    zchunk = std::max(1, (v.nz + nch - 1) / nch);
    if (zchunk < 16 && v.nz >= 16) zchunk = 16;
    if (zchunk > v.nz) zchunk = v.nz;
    items_per_box = (long long)ntiles * ((v.nz + zchunk - 1) / zchunk);
    items = items_per_box * nboxes;
    grid = (int)std::min<long long>(std::min<long long>(items, resident), max_grid);
}

static int64_t diag_scratch_bytes(int64_t ncell) { return 256 + (int64_t)diag_grid(ncell) * sizeof(DiagPartial); }

static int run_diag(const DiagView &v, const axs_diag_params *p, const uint8_t *mask, axs_diag_result *out,
                    int64_t *list, int64_t capacity, void *scratch, int64_t scratch_bytes, cudaStream_t st,
                    int nboxes = 1, int64_t box_stride = 0, uint8_t *tags = nullptr)
{
    AXS_REQUIRE(p != nullptr && out != nullptr, AXS_ERR_INVALID_ARGUMENT, "null params or result");
    AXS_REQUIRE(p->dx > 0.0 && p->R > 0.0 && p->m_r > 0.0, AXS_ERR_INVALID_ARGUMENT,
                "dx, R and m_r must be positive");
    AXS_REQUIRE(p->masking_scheme >= AXS_MASK_NONE && p->masking_scheme <= AXS_MASK_B, AXS_ERR_INVALID_ARGUMENT,
                "bad masking scheme %d", p->masking_scheme);
    AXS_REQUIRE(capacity >= 0, AXS_ERR_INVALID_ARGUMENT, "negative list capacity");
    AXS_REQUIRE(capacity == 0 || list != nullptr, AXS_ERR_INVALID_ARGUMENT, "null list with positive capacity");
    AXS_REQUIRE(nboxes >= 1, AXS_ERR_INVALID_ARGUMENT, "no boxes");
    const int64_t ncell = (int64_t)v.nx * v.ny * v.nz * nboxes;
    const int64_t need = diag_scratch_bytes(ncell);
    AXS_REQUIRE(scratch != nullptr && scratch_bytes >= need, AXS_ERR_WORKSPACE,
                "diagnostics scratch too small (%lld < %lld bytes)", (long long)scratch_bytes, (long long)need);
    AXS_REQUIRE(((uintptr_t)scratch % 16) == 0, AXS_ERR_ALIGNMENT, "scratch must be 16-byte aligned");
    DiagConst q{};
    q.one_over_dx = 1.0 / p->dx;
    q.R = p->R;
    q.R2 = p->R * p->R;
    q.inv_R = 1.0 / p->R;
    q.inv_R2 = 1.0 / q.R2;
    q.inv_R4 = q.inv_R2 * q.inv_R2;
    {
        // Velocity.hpp:62-78: term1 = |phi'|^2/(2 m^2 c1^2) (1 - e1 |phi|^2/c1^3),
        //                     term2 = e1/(4 m^2 c1^5) (phi . phi')^2
        const double c1 = 0.41222, e1 = -0.025763, m2 = p->m_r * p->m_r, c1s = c1 * c1;
        q.vel_a = 1.0 / (2.0 * m2 * c1s);
        q.vel_b = e1 / (c1 * c1s);
        q.vel_c = e1 / (4.0 * m2 * c1s * c1s * c1);
    }
    q.lambda = p->lambda;
    q.RpR = p->R_prime_over_R;
    q.m_r = p->m_r;
    q.threshold = p->masking_threshold;
    q.scheme = p->masking_scheme;
    q.want_energy = p->want_energy != 0;
    q.want_plaq = p->want_plaquettes != 0;
    q.want_vel = p->want_velocity != 0;
    q.f_one_over_dx = (float)q.one_over_dx;
    q.f_R2 = (float)q.R2;
    q.f_inv_R = (float)q.inv_R;
    q.f_inv_R2 = (float)q.inv_R2;
    q.f_inv_R4 = (float)q.inv_R4;
    q.f_lambda = (float)q.lambda;
    q.f_RpR = (float)q.RpR;
    q.f_threshold = (float)q.threshold;
    q.f_vel_a = (float)q.vel_a;
    q.f_vel_b = (float)q.vel_b;
    q.f_vel_c = (float)q.vel_c;
    auto *counter = static_cast<unsigned long long *>(scratch);
    auto *partials = reinterpret_cast<DiagPartial *>(static_cast<char *>(scratch) + 256);
    AXS_CUDA_CHECK(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st));
    int tiles_x, ntiles, zchunk, grid;
    long long items, items_per_box;
    long long *lst = (q.want_plaq && capacity > 0) ? reinterpret_cast<long long *>(list) : nullptr;
    int rc0 = AXS_OK;
    const bool offs31 = (int64_t)(v.ny + 2 * v.oy + 2) * v.js < INT_MAX;  // in-plane offsets in 31 bits
    auto launch_finder = [&](auto kern, int e_from) -> int {
        AXS_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FinderSmem)));
        kern<<<grid, kDiagThreads, sizeof(FinderSmem), st>>>(v, q, mask, partials, counter, lst, capacity, tiles_x,
                                                              ntiles, zchunk, items, items_per_box, box_stride, tags,
                                                              e_from);
        return launch_status("string finder");
    };
    if (q.want_plaq && !q.want_energy && !q.want_vel && offs31) {
        // windings only: the edge-code finder
        const bool f32 = v.dtype != AXS_F64;
        diag_plan(v, nboxes, diag_grid(ncell), FTX, FTY, f32 ? 4 : 3, tiles_x, ntiles, zchunk, items_per_box, items,
                  grid);
        rc0 = f32 ? launch_finder(finder_kernel<float, false>, 0) : launch_finder(finder_kernel<double, false>, 0);
        if (rc0) return rc0;
        diag_finalize_kernel<<<1, 256, 0, st>>>(partials, grid, counter, capacity, lst != nullptr, out);
        return launch_status("diagnostics finalize");
    }
    if (q.want_energy && v.dtype == AXS_F32 && p->per_cell_fp32 && offs31) {
        // per-cell FP32 terms: the energy sums (3 blocks per SM) and, over the same work
        // items, the windings, the list and the velocity (4 per SM). Each kernel fills
        // its own fields of the partial records; the finder clears the energy sums of
        // the records the energy kernel has no block for.
        const bool strings = q.want_plaq || q.want_vel;
        diag_plan(v, nboxes, diag_grid(ncell), FTX, FTY, q.want_vel ? 3 : 4, tiles_x, ntiles, zchunk, items_per_box,
                  items, grid);
        const int sms = device_sm_count() > 0 ? device_sm_count() : 148;
        const int egrid = strings ? std::min(grid, 3 * sms) : grid;
        AXS_CUDA_CHECK(
            cudaFuncSetAttribute(energy32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(EnergySmem)));
        energy32_kernel<<<egrid, kDiagThreads, sizeof(EnergySmem), st>>>(v, q, mask, partials, tiles_x, ntiles, zchunk,
                                                                          items, items_per_box, box_stride, !strings);
        if ((rc0 = launch_status("energy sums"))) return rc0;
        if (strings) {
            rc0 = q.want_vel ? launch_finder(finder_kernel<float, true>, egrid)
                             : launch_finder(finder_kernel<float, false>, egrid);
            if (rc0) return rc0;
        }
        diag_finalize_kernel<<<1, 256, 0, st>>>(partials, grid, counter, capacity, lst != nullptr, out);
        return launch_status("diagnostics finalize");
    }
    diag_plan(v, nboxes, diag_grid(ncell), DTX, DTY, 2, tiles_x, ntiles, zchunk, items_per_box, items, grid);
    auto launch = [&](auto kern, size_t smem) -> int {
        AXS_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<grid, kDiagThreads, smem, st>>>(v, q, mask, partials, counter, lst, capacity, tiles_x, ntiles, zchunk,
                                               items, items_per_box, box_stride, tags);
        return AXS_OK;
    };
    if (v.dtype == AXS_F64)
        rc0 = launch(diag_kernel<double, false>, sizeof(DiagSmem<double, false>));
    else if (p->per_cell_fp32)
        rc0 = launch(diag_kernel<float, true>, sizeof(DiagSmem<float, true>));
    else
        rc0 = launch(diag_kernel<float, false>, sizeof(DiagSmem<float, false>));
    if (rc0) return rc0;
    int rc = launch_status("diagnostics");
    if (rc) return rc;
    diag_finalize_kernel<<<1, 256, 0, st>>>(partials, grid, counter, capacity, lst != nullptr, out);
    return launch_status("diagnostics finalize");
}

// One periodic box in level layout (an ensemble member), without the pierced list.
int diag_level_box(const void *data, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g,
                   const axs_diag_params *p, axs_diag_result *out, void *scratch, int64_t scratch_bytes,
                   cudaStream_t st)
{
    DiagView v{data, dtype, nx, ny, nz, g.ox, g.oy, 0, 1, 1, 1, g.js, g.ks, g.cs};
    return run_diag(v, p, nullptr, out, nullptr, 0, scratch, scratch_bytes, st);
}

int64_t diag_scratch_bytes_for(int64_t ncell) { return diag_scratch_bytes(ncell); }

// The refinement tagger's plaquette criterion on a periodic level: the string
// finder's pass (same windings, bit for bit) writing one tag byte per cell
// (x fastest) instead of a pierced list. `out` is a device result record.
int diag_level_plaquette_tags(const void *state, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g, double dx,
                              uint8_t *tags, axs_diag_result *out, void *scratch, int64_t scratch_bytes,
                              cudaStream_t st)
{
    DiagView v{state, dtype, nx, ny, nz, g.ox, g.oy, 0, 1, 1, 1, g.js, g.ks, g.cs};
    axs_diag_params p{};
    p.dx = dx;
    p.R = 1.0;
    p.m_r = 1.0;
    p.masking_scheme = AXS_MASK_NONE;
    p.boundary = AXS_BOUNDARY_PERIODIC;
    p.want_plaquettes = 1;
    return run_diag(v, &p, nullptr, out, nullptr, 0, scratch, scratch_bytes, st, 1, 0, tags);
}

// nboxes boxes of one geometry, box_stride elements apart, with explicit ghost
// layers (refined patches), summed into one result. A pierced-list entry is
// 4 * (q * nx * ny * nz + cell) + plane for box q.
int diag_ghost_boxes(const void *data, int32_t dtype, int nx, int ny, int nz, int ox, int oy, int oz, int64_t js,
                     int64_t ks, int64_t cs, int nboxes, int64_t box_stride, const axs_diag_params *p,
                     axs_diag_result *out, int64_t *list, int64_t capacity, void *scratch, int64_t scratch_bytes,
                     cudaStream_t st)
{
    DiagView v{data, dtype, nx, ny, nz, ox, oy, oz, 0, 0, 0, js, ks, cs};
    return run_diag(v, p, nullptr, out, list, capacity, scratch, scratch_bytes, st, nboxes, box_stride);
}

}  // namespace axs

using namespace axs;

extern "C" {

int axs_diagnostics_scratch_bytes(int32_t nx, int32_t ny, int32_t nz, int64_t *bytes)
{
    AXS_REQUIRE(bytes != nullptr, AXS_ERR_INVALID_ARGUMENT, "null output");
    AXS_REQUIRE(nx > 0 && ny > 0 && nz > 0, AXS_ERR_INVALID_ARGUMENT, "empty box");
    *bytes = diag_scratch_bytes((int64_t)nx * ny * nz);
    return AXS_OK;
}

int axs_diagnostics(const axs_fab *state, const axs_diag_params *p, const uint8_t *mask, axs_diag_result *out,
                    int64_t *list, int64_t capacity, void *scratch, int64_t scratch_bytes, void *stream)
{
    AXS_REQUIRE(p != nullptr, AXS_ERR_INVALID_ARGUMENT, "null params");
    const int periodic = p->boundary == AXS_BOUNDARY_PERIODIC;
    AXS_REQUIRE(p->boundary == AXS_BOUNDARY_GHOSTS || periodic, AXS_ERR_INVALID_ARGUMENT, "bad boundary mode");
    const int need_ng = periodic ? 0 : (p->want_energy ? 2 : 1);
    int rc = validate_fab(state, "state", 4, need_ng);
    if (rc) return rc;
    DiagView v{state->data, state->dtype, state->nx, state->ny, state->nz, state->ng, state->ng, state->ng,
               periodic, periodic, periodic, state->jstride, state->kstride, state->cstride};
    return run_diag(v, p, mask, out, list, capacity, scratch, scratch_bytes, (cudaStream_t)stream);
}

int axs_level_diagnostics(const axs_level *lv, const axs_diag_params *p, const uint8_t *mask, axs_diag_result *out,
                          int64_t *list, int64_t capacity, void *scratch, int64_t scratch_bytes, void *stream)
{
    LevelGeom g;
    AXS_REQUIRE(lv != nullptr && lv->state != nullptr, AXS_ERR_INVALID_ARGUMENT, "null level");
    int rc = level_geom(lv->dtype, lv->nx, lv->ny, lv->nz, g);
    if (rc) return rc;
    // indices wrap on every axis: the sweeps keep the x/y padding current but
    // not its corners, which the xy plaquette at (nx-1, ny-1) would read
    DiagView v{lv->state, lv->dtype, lv->nx, lv->ny, lv->nz, g.ox, g.oy, 0, 1, 1, 1, g.js, g.ks, g.cs};
    return run_diag(v, p, mask, out, list, capacity, scratch, scratch_bytes, (cudaStream_t)stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Diagnostics without caller-provided scratch.
//
// Some host codes cannot hand this library any extra device memory: an AMReX
// application, for instance, gives most of the GPU to its own arena at start-up
// and expects plugins to work inside the buffers they are passed, and other
// callers run under a fixed device-memory budget where a cudaMalloc from a
// plugin is not allowed. For them the diagnostics pass can use the scratch
// array below, a file-scope device array that every GPU loading this library
// holds until the process exits. Its size caps the per-block partials the pass
// needs (256 bytes of header + 160 bytes per block); on a 152-SM GB300 a pass
// uses at most 1216 blocks, i.e. about 195 KB of the 256 KiB.
namespace axs {
constexpr size_t kStaticDiagScratchBytes = 256 * 1024;
static __device__ __align__(256) unsigned char g_static_diag_scratch[kStaticDiagScratchBytes];

// Device address of g_static_diag_scratch, looked up once per device with that
// device current (host code must not use the symbol itself as an address).
static int static_scratch_address(void **out)
{
    constexpr int kMaxDevices = 64;
    static void *addr[kMaxDevices] = {};
    static std::mutex mu;
    int dev = 0;
    AXS_CUDA_CHECK(cudaGetDevice(&dev));
    AXS_REQUIRE(dev >= 0 && dev < kMaxDevices, AXS_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(mu);
    if (addr[dev] == nullptr) {
        void *p = nullptr;
        AXS_CUDA_CHECK(cudaGetSymbolAddress(&p, g_static_diag_scratch));
        addr[dev] = p;
    }
    *out = addr[dev];
    return AXS_OK;
}
}  // namespace axs

extern "C" {

int axs_diagnostics_static_scratch(const axs_fab *state, const axs_diag_params *p, const uint8_t *mask,
                                   axs_diag_result *result_dev, int64_t *pierced_dev, int64_t pierced_capacity,
                                   void *stream)
{
    AXS_REQUIRE(state != nullptr, AXS_ERR_INVALID_ARGUMENT, "null state");
    const int64_t ncell = (int64_t)state->nx * state->ny * state->nz;
    AXS_REQUIRE(ncell > 0, AXS_ERR_INVALID_ARGUMENT, "empty box");
    const int64_t need = diag_scratch_bytes(ncell);
    AXS_REQUIRE(need <= (int64_t)kStaticDiagScratchBytes, AXS_ERR_WORKSPACE,
                "diagnostics needs %lld scratch bytes on this device, more than the %lld-byte static array; "
                "use axs_diagnostics with caller-provided scratch",
                (long long)need, (long long)kStaticDiagScratchBytes);
    void *scratch = nullptr;
    int rc = static_scratch_address(&scratch);
    if (rc) return rc;
    // run_diag clears the list counter in the array before the pass; the
    // per-block partials are overwritten in full.
    return axs_diagnostics(state, p, mask, result_dev, pierced_dev, pierced_capacity, scratch,
                           (int64_t)kStaticDiagScratchBytes, stream);
}

}  // extern "C"
