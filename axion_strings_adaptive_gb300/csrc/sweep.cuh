// Generic TMA-staged stencil sweep over a periodic level (sm_103a).
//
// A sweep reads four components of one level-layout array with the 13-point
// 4th-order star (their Laplacians and centre values) plus up to 12 components
// of other level-layout arrays pointwise, and hands both to a per-site
// operation that writes its outputs. The forward RK4 sweeps and the two
// adjoint sweeps are such operations (rk4_level.cu, adjoint.cu).
//
// Pipeline: a block owns a TX x TY tile of the xy plane over a chunk of z
// planes and marches in z. One elected thread issues one 4D TMA load per plane
// ({x, y, z, component} box of (TX+8) x (TY+4) x 1 x 4) into an NS-slot
// shared-memory ring; completion is signalled through one mbarrier per slot and
// every wait is bounded. Pointwise components are loaded one plane ahead into
// registers. Work items (tile, z-chunk) are numbered tile-fastest so the blocks
// resident at any moment work on neighbouring tiles of the same z range.
//
// A work item belongs to a box: the one level of a single-level sweep, or one
// of many independent levels packed component-major in one arena (an ensemble,
// ensemble.cu), each box then having its own tensor map and offset in every
// component plane. The work-item source is a template policy, so the
// single-level kernel reads its geometry from the launch parameters.
#pragma once

#include <algorithm>
#include <type_traits>

#include "axs_internal.cuh"

namespace axs {

template <typename T> struct StageCoef {
    T kappa, hlam, R2;  // kappa, lambda/2, R^2 at one stage time
};

constexpr int kMaxPointwise = 12;

template <typename T> struct SweepArgs {
    int nx, ny, nz;
    int tiles_x, ntiles, zchunk;
    int64_t n_items;
    int64_t js, ks, cs;
    int ox;                      // x offset of the valid region in a padded row of the stencil arrays
    int dox_pt, dox_out;         // element offset of the pointwise inputs / the outputs relative to the
                                 // stencil arrays' layout (0 unless their rows are shifted, refined patches)
    T wA, wB, wC;                // lap = wA*S1 + wB*S2 + wC*f0 (S1/S2: sums of +-1 / +-2 neighbours)
    StageCoef<T> c1, c2, c4;     // stage coefficients at t, t + h/2, t + h
    T h, h_half, h2_quarter, h2_half, h_sixth, h_third, h2_sixth;
    // remainders of the FP32 weights and step fractions (exact value - FP32 value),
    // used by the compensated FP32 step
    T wA_lo, wB_lo, h_lo, h_half_lo, h2_quarter_lo, h2_half_lo, h_sixth_lo, h_third_lo, h2_sixth_lo;
    const T *pt[kMaxPointwise];  // pointwise input components (level layout)
    T *out[8];                   // output components (level layout)
    double inv_lambda0;          // adjoint: dlambda_s/dlambda0 = lambda_s / lambda0
    double *lam_partial;         // adjoint: one lambda0-gradient partial per block
    unsigned *status;
    uint32_t wait_polls;         // polls before a bounded wait gives up (device_wait_polls at launch)
    // box-table sweeps: box table, packed work items (box << 16 | item in box),
    // two tensor maps per box (state, stage buffers) and which one this sweep reads
    const struct EnsBoxDesc *boxes;
    const uint32_t *items;
    const CUtensorMap *maps;
    int map_sel;
};

// One box of a box table (device table entry): an ensemble member, or the
// sweep domain of one refined patch. Element offsets are relative to the arena
// base of each component plane. The sweep covers the domain
// [xlo, xlo+nx) x [ylo, ylo+ny) x [zlo, zlo+nz) (box coordinates, valid cell
// (0,0,0) at padded position (ox, oy, oz)); periodic boxes wrap z by plane
// index and write periodic copies, patches read and write explicit ghost rings.
struct EnsBoxDesc {
    int nx, ny, nz;
    int tiles_x, ntiles, zchunk;
    int64_t js, ks;
    int64_t base;  // element offset of the box's (padded) origin in every component plane
    int xlo, ylo, zlo;
    int oy, oz;    // padded row / plane of valid y = 0 / z = 0
    int periodic;  // 1: wrap z, write periodic copies; 0: explicit ghost rings
    int map_box;   // two-sweep tensor maps 2*map_box (state), 2*map_box + 1 (stage buffers);
                   // an ensemble's fused step uses maps 6*map_box .. 6*map_box + 5
    int pad;
};
constexpr int kEnsItemBits = 16;  // work items per box < 2^16; boxes < 2^16

// Geometry of the box a work item belongs to, and the item's number in it.
struct BoxGeom {
    int nx, ny, nz;
    int tiles_x, ntiles, zchunk;
    int64_t js, ks, base;
    const CUtensorMap *map;
    int64_t local;
    int xlo, ylo, zlo, oy, oz;
    bool periodic;
};

// Work-item sources.
struct SingleLevel {  // the one periodic level described by the launch parameters
    template <typename T>
    __device__ __forceinline__ static BoxGeom item(const SweepArgs<T> &a, const CUtensorMap *map, int64_t it)
    {
        return BoxGeom{a.nx, a.ny, a.nz, a.tiles_x, a.ntiles, a.zchunk, a.js, a.ks, 0, map, it, 0, 0, 0, 2, 0, true};
    }
};
struct BoxTable {  // the boxes of an ensemble, or the patches of a refined level
    template <typename T>
    __device__ __forceinline__ static BoxGeom item(const SweepArgs<T> &a, const CUtensorMap *, int64_t it)
    {
        const uint32_t e = __ldg(a.items + it);
        const int b = (int)(e >> kEnsItemBits);
        const EnsBoxDesc &d = a.boxes[b];
        return BoxGeom{d.nx,    d.ny,     d.nz,
                       d.tiles_x, d.ntiles, d.zchunk,
                       d.js,    d.ks,     d.base,
                       a.maps + 2 * d.map_box + a.map_sel, (int64_t)(e & ((1u << kEnsItemBits) - 1)),
                       d.xlo,   d.ylo,    d.zlo,
                       d.oy,    d.oz,     d.periodic != 0};
    }
};

template <typename T, int V, int TX, int TY> struct SweepShape {
    static constexpr int NTX = TX / V;
    static constexpr int NT = NTX * TY;
    static constexpr int BX = TX + 8;
    static constexpr int BY = TY + 4;
    static constexpr int TILE = BX * BY;
    static constexpr int SLOT = 4 * TILE;
    static constexpr uint32_t SLOT_BYTES = SLOT * sizeof(T);
    static constexpr int PRE = (2 + V - 1) / V;  // vectors left/right of the centre that cover +-2
    static constexpr int NROW = 2 * PRE + 1;
    static_assert(TX % V == 0 && 4 % V == 0, "tile width and halo must hold whole vectors");
    static_assert((BX * sizeof(T)) % 16 == 0, "TMA box row must be a multiple of 16 bytes");
    static_assert(SLOT_BYTES % 128 == 0, "ring slots must stay 128-byte aligned");
    static_assert(BX <= 256 && BY <= 256, "TMA box extent limit");
};

// One output vector: a plain store, or (HINT) one with an L2 policy.
template <typename T, int V, bool HINT>
__device__ __forceinline__ void st_out(T *p, const T *v, uint64_t pol)
{
    if constexpr (HINT)
        stv_hint<T, V>(p, v, pol);
    else
        stv<T, V>(p, v);
}

// Store V sites and, for sites next to the domain edge, their periodic copies
// in the x/y padding (8 columns, 2 rows, and the corners where both meet).
// The sweeps' stencils read 4 padding columns; 8 fill whole 32-byte sectors
// (FP32; two for FP64), since a partly written sector costs a DRAM read on top
// of its write. The one-pass level step reads all 8 columns and the corners.
template <typename T, int V, bool HINT = false>
__device__ __forceinline__ void store_with_copies(T *base, int64_t off, int x, int y, int nx, int ny, int64_t js,
                                                  const T *v, uint64_t pol = 0, bool periodic = true)
{
    st_out<T, V, HINT>(base + off, v, pol);
    if (!periodic) return;
    const bool xl = x < 8, xh = x >= nx - 8;
    const int64_t sy = (int64_t)ny * js;
    if (xl) st_out<T, V, HINT>(base + off + nx, v, pol);
    if (xh) st_out<T, V, HINT>(base + off - nx, v, pol);
    if (y < 2) {
        st_out<T, V, HINT>(base + off + sy, v, pol);
        if (xl) st_out<T, V, HINT>(base + off + sy + nx, v, pol);
        if (xh) st_out<T, V, HINT>(base + off + sy - nx, v, pol);
    }
    if (y >= ny - 2) {
        st_out<T, V, HINT>(base + off - sy, v, pol);
        if (xl) st_out<T, V, HINT>(base + off - sy + nx, v, pol);
        if (xh) st_out<T, V, HINT>(base + off - sy - nx, v, pol);
    }
}

// Two FP32 sites per instruction: Blackwell's packed FP32x2 add, multiply and
// fused multiply-add (__fadd2_rn, __fmul2_rn, __ffma2_rn; each lane rounds as
// the scalar instruction does). A thread's V sites are consecutive in x, so a
// pair of them is one F2. Differences are sums with a negated operand, which is
// exact, so every expression below rounds exactly as its scalar form.
using ::fma;  // the scalar overloads stay visible next to the F2 one below
struct F2 {
    float2 v;
    __device__ __forceinline__ F2() {}
    __device__ __forceinline__ F2(float a, float b) : v(make_float2(a, b)) {}
    __device__ __forceinline__ explicit F2(float a) : v(make_float2(a, a)) {}
    __device__ __forceinline__ explicit F2(float2 a) : v(a) {}
};
__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return F2(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return F2(__fadd2_rn(a.v, make_float2(-b.v.x, -b.v.y))); }
__device__ __forceinline__ F2 operator*(F2 a, F2 b) { return F2(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ F2 fma(F2 a, F2 b, F2 c) { return F2(__ffma2_rn(a.v, b.v, c.v)); }

// FP32 with an even number of sites per thread goes through F2 pairs.
template <typename T, int V> constexpr bool kPackedPairs = std::is_same<T, float>::value && V % 2 == 0;

// F(u) = lap + (kappa - lambda/2 (|u|^2 - R^2)) u, one component pair.
template <typename T>
__device__ __forceinline__ void rhs_pair(const StageCoef<T> &c, T u1, T u2, T l1, T l2, T &f1, T &f2)
{
    const T k = fma(-c.hlam, fma(u1, u1, u2 * u2) - c.R2, c.kappa);
    f1 = fma(k, u1, l1);
    f2 = fma(k, u2, l2);
}

// the same for two sites at once
__device__ __forceinline__ void rhs_pair(const StageCoef<float> &c, F2 u1, F2 u2, F2 l1, F2 l2, F2 &f1, F2 &f2)
{
    const F2 k = fma(F2(-c.hlam), fma(u1, u1, u2 * u2) + F2(-c.R2), F2(c.kappa));
    f1 = fma(k, u1, l1);
    f2 = fma(k, u2, l2);
}

// J_F(u)^T a = lap(a) + kappa a - lambda/2 [(|u|^2 - R^2) a + 2 u (u . a)]
template <typename T>
__device__ __forceinline__ void rhs_adjoint_pair(const StageCoef<T> &c, T u1, T u2, T a1, T a2, T la1, T la2, T &o1,
                                                 T &o2)
{
    const T m = fma(u1, u1, u2 * u2) - c.R2;
    const T k = fma(-c.hlam, m, c.kappa);
    const T ua = T(2) * c.hlam * fma(u1, a1, u2 * a2);
    o1 = fma(k, a1, la1) - ua * u1;
    o2 = fma(k, a2, la2) - ua * u2;
}

// The FP32 Laplacian of two neighbouring sites x, x+1 from their neighbours:
// r[0..5] = f(x-2 .. x+3) along the row, and the y / z neighbour pairs. The
// stencil as differences from the centre, lap = wA sum(f+-1 - f0) + wB
// sum(f+-2 - f0): a neighbour within a factor 2 of f0 gives an exact
// difference, so the -30 f0 term of the plain sum does not cancel against the
// neighbours. f - f0 is formed as f + (-f0), the same IEEE result. Every FP32
// sweep evaluates its stencils through this function. COMP (the compensated
// FP32 step) adds the weights' FP32 remainders times d1, d2: FP32 rounds 16/3
// and -1/3 in the same direction for every site, a bias that the plain form
// carries into every step.
template <bool COMP = false>
__device__ __forceinline__ void lap_pair(const SweepArgs<float> &a, const float *r, float2 ym1, float2 yp1,
                                         float2 ym2, float2 yp2, float2 zm1, float2 zp1, float2 zm2, float2 zp2,
                                         float &l0, float &l1)
{
    const F2 m0(-r[2], -r[3]);
    const F2 d1 = ((F2(r[1], r[2]) + m0) + (F2(r[3], r[4]) + m0)) + ((F2(ym1) + m0) + (F2(yp1) + m0)) +
                  ((F2(zm1) + m0) + (F2(zp1) + m0));
    const F2 d2 = ((F2(r[0], r[1]) + m0) + (F2(r[4], r[5]) + m0)) + ((F2(ym2) + m0) + (F2(yp2) + m0)) +
                  ((F2(zm2) + m0) + (F2(zp2) + m0));
    F2 l = fma(F2(a.wA), d1, F2(a.wB) * d2);
    if constexpr (COMP) l = fma(F2(a.wA_lo), d1, fma(F2(a.wB_lo), d2, l));  // the weights' FP32 remainders
    l0 = l.v.x;
    l1 = l.v.y;
}

// The 13-point 4th-order Laplacian and the centre values of V consecutive
// sites of one component, from five z planes held in shared memory (planes
// z-2 .. z+2; `at` is the first site's element offset in a plane, `bx` the row
// length). Every sweep evaluates its stencils through this function, so all of
// them round alike. FP32: differences from the centre first (exact while a
// neighbour lies within a factor 2 of f0), so the -30 f0 term of the stencil
// does not cancel against the neighbour sums: lap = wA sum(f+-1 - f0) +
// wB sum(f+-2 - f0), two sites per packed instruction where V is even. FP64:
// the plain weighted sums.
template <typename T, int V, bool COMP = false>
__device__ __forceinline__ void star_laplacian(const SweepArgs<T> &a, const T *zm2p, const T *zm1p, const T *P0,
                                               const T *zp1p, const T *zp2p, int at, int bx, T (&lap)[V],
                                               T (&ctr)[V])
{
    constexpr int PRE = (2 + V - 1) / V, NROW = 2 * PRE + 1;
    T row[NROW * V], ym1[V], yp1[V], ym2[V], yp2[V], zm1[V], zp1[V], zm2[V], zp2[V];
#pragma unroll
    for (int r = 0; r < NROW; ++r) ldv<T, V>(P0 + at + (r - PRE) * V, row + r * V);
    ldv<T, V>(P0 + at - bx, ym1);
    ldv<T, V>(P0 + at + bx, yp1);
    ldv<T, V>(P0 + at - 2 * bx, ym2);
    ldv<T, V>(P0 + at + 2 * bx, yp2);
    ldv<T, V>(zm1p + at, zm1);
    ldv<T, V>(zp1p + at, zp1);
    ldv<T, V>(zm2p + at, zm2);
    ldv<T, V>(zp2p + at, zp2);
    if constexpr (kPackedPairs<T, V>) {
#pragma unroll
        for (int v = 0; v < V; v += 2) {
            const int ci = PRE * V + v;
            lap_pair<COMP>(a, row + ci - 2, make_float2(ym1[v], ym1[v + 1]), make_float2(yp1[v], yp1[v + 1]),
                     make_float2(ym2[v], ym2[v + 1]), make_float2(yp2[v], yp2[v + 1]), make_float2(zm1[v], zm1[v + 1]),
                     make_float2(zp1[v], zp1[v + 1]), make_float2(zm2[v], zm2[v + 1]), make_float2(zp2[v], zp2[v + 1]),
                     lap[v], lap[v + 1]);
            ctr[v] = row[ci];
            ctr[v + 1] = row[ci + 1];
        }
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int ci = PRE * V + v;
            const T f0 = row[ci];
            if constexpr (std::is_same<T, float>::value) {
                const T d1 = ((row[ci - 1] - f0) + (row[ci + 1] - f0)) + ((ym1[v] - f0) + (yp1[v] - f0)) +
                             ((zm1[v] - f0) + (zp1[v] - f0));
                const T d2 = ((row[ci - 2] - f0) + (row[ci + 2] - f0)) + ((ym2[v] - f0) + (yp2[v] - f0)) +
                             ((zm2[v] - f0) + (zp2[v] - f0));
                lap[v] = fma(a.wA, d1, a.wB * d2);
                if constexpr (COMP) lap[v] = fma(a.wA_lo, d1, fma(a.wB_lo, d2, lap[v]));
            } else {
                const T s1 = (row[ci - 1] + row[ci + 1]) + (ym1[v] + yp1[v]) + (zm1[v] + zp1[v]);
                const T s2 = (row[ci - 2] + row[ci + 2]) + (ym2[v] + yp2[v]) + (zm2[v] + zp2[v]);
                lap[v] = fma(a.wA, s1, fma(a.wB, s2, a.wC * f0));
            }
            ctr[v] = f0;
        }
    }
}

// The lambda0-gradient sum of an adjoint sweep: per thread in the field
// precision with Neumaier compensation, widened to double once for the block
// sum (a conversion and an FP64 add per site run at GB300's FP64 rate).
template <typename T> struct LamAcc {
    T s = T(0), c = T(0);
    __device__ __forceinline__ void add(T x)
    {
        const T t = s + x;
        c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

template <typename T, int V, int TX, int TY, int NS, int MINB, class Op, class Src = SingleLevel, bool HINT = false>
__global__ void __launch_bounds__(SweepShape<T, V, TX, TY>::NT, MINB)
    stencil_sweep_kernel(const __grid_constant__ CUtensorMap tmap, const SweepArgs<T> a)
{
    using S = SweepShape<T, V, TX, TY>;
    constexpr int NPT = Op::kPointwise;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *ring = reinterpret_cast<T *>(smem_raw);
    __shared__ uint64_t full[NS];
    __shared__ double lam_red[(S::NT + 31) / 32];

    const int tid = threadIdx.x;
    const int tx = tid % S::NTX, ty = tid / S::NTX;
    LamAcc<T> lam_acc;
    // HINT: stencil planes (re-read by neighbouring tiles) evict-last in L2,
    // pointwise inputs and all outputs (touched once) evict-first
    const uint64_t pol_first = HINT ? l2_policy_evict_first() : 0, pol_last = HINT ? l2_policy_evict_last() : 0;

    if (tid == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
        if constexpr (std::is_same<Src, SingleLevel>::value) prefetch_tensormap(&tmap);
    }
    __syncthreads();

    // ---- producer cursor (thread 0 only) ----
    int64_t p_item = blockIdx.x;
    int p_k = 0, p_len = 0, p_za = 0, p_nz = 1, p_x = 0, p_y = 0;
    const CUtensorMap *p_map = &tmap;
    int p_oy = 2, p_oz = 0;
    bool p_wrap = true;
    auto p_start = [&]() {
        if (p_item >= a.n_items) return;
        const BoxGeom b = Src::item(a, &tmap, p_item);
        const int tile = (int)(b.local % b.ntiles);
        const int c0 = (int)(b.local / b.ntiles) * b.zchunk;
        p_za = b.zlo + c0;
        p_len = min(b.zchunk, b.nz - c0);
        p_nz = b.nz;
        p_x = b.xlo + (tile % b.tiles_x) * TX;
        p_y = b.ylo + (tile / b.tiles_x) * TY;
        p_oy = b.oy;
        p_oz = b.oz;
        p_wrap = b.periodic;
        p_map = b.map;
        if constexpr (!std::is_same<Src, SingleLevel>::value) fence_tensormap_acquire(p_map);
    };
    int64_t q_issued = 0;
    auto issue_one = [&]() -> bool {
        if (p_item >= a.n_items) return false;
        int zp = p_za - 2 + p_k;
        if (p_wrap) {
            zp %= p_nz;
            if (zp < 0) zp += p_nz;
        } else {
            zp += p_oz;  // explicit ghost planes: padded plane index, no wrap
        }
        const int slot = (int)(q_issued % NS);
        mbar_arrive_expect_tx(&full[slot], S::SLOT_BYTES);
        // box x starts 4 columns left of the tile: padded column ox + x0 - 4 (16-byte aligned);
        // box y starts 2 rows above the tile: padded row y0 - 2 + oy
        if constexpr (HINT)
            tma_load_4d_hint(ring + (size_t)slot * S::SLOT, p_map, a.ox - 4 + p_x, p_y - 2 + p_oy, zp, 0, &full[slot],
                             pol_last);
        else
            tma_load_4d(ring + (size_t)slot * S::SLOT, p_map, a.ox - 4 + p_x, p_y - 2 + p_oy, zp, 0, &full[slot]);
        ++q_issued;
        if (++p_k == p_len + 4) {
            p_k = 0;
            p_item += gridDim.x;
            p_start();
        }
        return true;
    };
    if (tid == 0) {
        p_start();
        for (int s = 0; s < NS; ++s)
            if (!issue_one()) break;
    }

    int64_t q_base = 0, q_waited = 0;
    bool aborted = false;
    const int xl = 4 + V * tx;  // tile-local column of this thread's first site
    const int yl = 2 + ty;
    for (int64_t item = blockIdx.x; item < a.n_items; item += gridDim.x) {
        const BoxGeom b = Src::item(a, &tmap, item);
        const int tile = (int)(b.local % b.ntiles);
        const int c0 = (int)(b.local / b.ntiles) * b.zchunk;
        const int za = b.zlo + c0;
        const int len = min(b.zchunk, b.nz - c0);
        const int x = b.xlo + (tile % b.tiles_x) * TX + V * tx;
        const int y = b.ylo + (tile / b.tiles_x) * TY + ty;
        const bool active = (x < b.xlo + b.nx) && (y < b.ylo + b.ny);
        // pointwise components of the next plane, loaded one iteration ahead
        T pn[NPT > 0 ? NPT : 1][V];
        if constexpr (NPT > 0) {
            if (active) {
                const int64_t off0 =
                    b.base + (int64_t)(x + a.ox) + (int64_t)(y + b.oy) * b.js + (int64_t)(za + b.oz) * b.ks;
#pragma unroll
                for (int c = 0; c < NPT; ++c) {
                    if constexpr (HINT)
                        ldv_nc_hint<T, V>(a.pt[c] + off0 + a.dox_pt, pn[c], pol_first);
                    else
                        ldv_nc<T, V>(a.pt[c] + off0 + a.dox_pt, pn[c]);
                }
            }
        }
        for (int m = 0; m < len; ++m) {
            const int z = za + m;
            const int64_t off = b.base + (int64_t)(x + a.ox) + (int64_t)(y + b.oy) * b.js + (int64_t)(z + b.oz) * b.ks;

            T pq[NPT > 0 ? NPT : 1][V];
            if constexpr (NPT > 0) {
#pragma unroll
                for (int c = 0; c < NPT; ++c)
#pragma unroll
                    for (int v = 0; v < V; ++v) pq[c][v] = pn[c][v];
                if (active && m + 1 < len) {
#pragma unroll
                    for (int c = 0; c < NPT; ++c) {
                        if constexpr (HINT)
                            ldv_nc_hint<T, V>(a.pt[c] + off + b.ks + a.dox_pt, pn[c], pol_first);
                        else
                            ldv_nc<T, V>(a.pt[c] + off + b.ks + a.dox_pt, pn[c]);
                    }
                }
            }

            const int64_t need = q_base + m + 4;
            bool late = false;  // this thread's wait expired
            while (q_waited <= need) {
                const int slot = (int)(q_waited % NS);
                if (!mbar_wait_bounded(&full[slot], (uint32_t)((q_waited / NS) & 1), a.wait_polls)) {
                    atomicOr(a.status, kDevTimeout);
                    late = true;
                }
                ++q_waited;
            }

            const T *sl[5];
#pragma unroll
            for (int d = 0; d < 5; ++d) sl[d] = ring + (size_t)((q_base + m + d) % NS) * S::SLOT;

            if (active) {
                T lap[4][V], ctr[4][V];
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    star_laplacian<T, V, Op::kComp>(a, sl[0] + c * S::TILE, sl[1] + c * S::TILE, sl[2] + c * S::TILE,
                                         sl[3] + c * S::TILE, sl[4] + c * S::TILE, yl * S::BX + xl, S::BX, lap[c],
                                         ctr[c]);
                Op::template apply<T, V, HINT>(a, b, lap, ctr, pq, off + a.dox_out, x, y, lam_acc, pol_first);
            }

            // everyone is done with the oldest plane of this window; the barrier
            // also ORs the threads' expired waits (the block stops after this plane)
            if (__syncthreads_or(late)) {
                aborted = true;
                break;
            }
            const int64_t next_needed = (m + 1 < len) ? (q_base + m + 1) : (q_base + len + 4);
            if (tid == 0) {
                fence_proxy_async_smem();
                while (q_issued < next_needed + NS && issue_one()) {
                }
            }
        }
        if (aborted) break;
        q_base += len + 4;
    }
    // A wait expired: make sure no bulk copy is still landing in shared memory
    // before the block exits (bounded as well).
    if (aborted && tid == 0) {
        for (int64_t q = q_waited; q < q_issued; ++q) mbar_wait_bounded(&full[q % NS], (uint32_t)((q / NS) & 1), 1u << 20);
    }
    if constexpr (Op::kLambdaGrad) {
        // fixed-order block reduction of the lambda0-gradient contributions
        double lv = lam_acc.value();
        for (int o = 16; o > 0; o >>= 1) lv += __shfl_down_sync(0xffffffffu, lv, o);
        if ((tid & 31) == 0) lam_red[tid >> 5] = lv;
        __syncthreads();
        if (tid == 0) {
            double s = 0.0;
            for (int w = 0; w < (S::NT + 31) / 32; ++w) s += lam_red[w];
            a.lam_partial[blockIdx.x] = s * a.inv_lambda0;
        }
    }
}

// Host: chunk length balancing the last wave against the 4 warm-up planes
// each chunk costs, while keeping the SMs busy.
inline void plan_chunks(int ntiles, int nz, int grid_cap, int &zchunk, int64_t &items, int &grid)
{
    double best = -1.0;
    zchunk = nz;
    for (int nch = 1; nch <= nz; ++nch) {
        const int lz = (nz + nch - 1) / nch;
        if ((nz + lz - 1) / lz != nch) continue;
        const int64_t it = (int64_t)ntiles * nch;
        const int g = (int)std::min<int64_t>(it, grid_cap);
        const int64_t waves = (it + g - 1) / g;
        const double fill = (double)it / (double)(waves * g);
        const double warm = (double)lz / (double)(lz + 4);
        const double par = (double)g / (double)grid_cap;
        const double score = fill * warm * std::min(1.0, par * 1.25);
        if (score > best + 1e-9) {
            best = score;
            zchunk = lz;
        }
    }
    items = (int64_t)ntiles * ((nz + zchunk - 1) / zchunk);
    grid = (int)std::min<int64_t>(items, grid_cap);
}

// One tiling of one sweep operation: occupancy, chunk plan and launch.
template <typename T, int V, int TX, int TY, int NS, int MINB, class Op, class Src = SingleLevel, bool HINT = false>
struct SweepLauncher {
    using S = SweepShape<T, V, TX, TY>;
    static size_t smem() { return (size_t)NS * S::SLOT_BYTES; }

    static int blocks_per_sm(int &bps)
    {
        static int cached = -1;
        if (cached < 0) {
            auto kern = stencil_sweep_kernel<T, V, TX, TY, NS, MINB, Op, Src, HINT>;
            AXS_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem()));
            int b = 0;
            AXS_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, S::NT, smem()));
            cached = std::max(1, b);
        }
        bps = cached;
        return AXS_OK;
    }

    // Fill the geometry part of `a` and return the grid size.
    static int plan(SweepArgs<T> &a, int nx, int ny, int nz, int &grid)
    {
        int bps = 0;
        int rc = blocks_per_sm(bps);
        if (rc) return rc;
        const int sms = device_sm_count();
        AXS_REQUIRE(sms > 0, AXS_ERR_CUDA, "no CUDA device");
        a.nx = nx;
        a.ny = ny;
        a.nz = nz;
        a.tiles_x = (nx + TX - 1) / TX;
        a.ntiles = a.tiles_x * ((ny + TY - 1) / TY);
        plan_chunks(a.ntiles, nz, bps * sms, a.zchunk, a.n_items, grid);
        return AXS_OK;
    }

    static int launch(const CUtensorMap &map, const SweepArgs<T> &a, int grid, cudaStream_t st)
    {
        stencil_sweep_kernel<T, V, TX, TY, NS, MINB, Op, Src, HINT><<<grid, S::NT, smem(), st>>>(map, a);
        return launch_status("stencil sweep");
    }

    static uint32_t box_x() { return S::BX; }
    static uint32_t box_y() { return S::BY; }
};

}  // namespace axs
