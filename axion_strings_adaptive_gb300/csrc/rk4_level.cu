// Fused classic-RK4 level advance: two TMA-staged stencil sweeps per step.
//
// Classic RK4 applied to y = (psi, Pi), y' = (Pi, F(t, psi)) with
//   F(t, psi) = lap(psi) + [kappa(t) - lambda(t)/2 (|psi|^2 - R(t)^2)] psi
// (AxionStringsRHS.impl.hpp:44-59) has stage states whose psi parts are
//   psi_n, psi_n + h/2 Pi_n, psi_n + h/2 Pi_n + h^2/4 F1, psi_n + h Pi_n + h^2/2 F2
// so the four stage RHS evaluations pair up:
//   sweep A reads (psi_n, Pi_n) and evaluates F1 = F(t, psi_n),
//                                             F2 = F(t+h/2, psi_n + h/2 Pi_n);
//   sweep B reads (S3, S4)      and evaluates F3 = F(t+h/2, S3), F4 = F(t+h, S4),
// with S3 = psi_n + h/2 Pi_n + h^2/4 F1, S4 = psi_n + h Pi_n + h^2/2 F2 and
//   psi_{n+1} = S4 + h^2/6 (F1 - 2 F2 + F3),
//   Pi_{n+1}  = [Pi_n + h/6 F1 + h/3 F2] + h/3 F3 + h/6 F4,
// which is classic RK4 term for term (exact arithmetic). Per site and step
// the sweeps move 4+8 and 8+4 words: 24 words instead of the 64 of a
// stage-by-stage three-register RK4.
//
// Each sweep is a persistent kernel. A block owns a TX x TY tile of the xy
// plane over a chunk of z planes and marches in z. One elected thread issues
// one 4D TMA load per plane ({x, y, z, component} box of (TX+8) x (TY+4) x 1 x 4,
// the 4 stencil components at once) into an NS-slot shared-memory ring,
// completion signalled through an mbarrier per slot; all waits are bounded.
// Each thread owns V consecutive x sites of one row. Periodic halos in x/y
// come from padding columns/rows that every sweep rewrites when it writes a
// boundary site; z wraps by plane index. Work items (tile, z-chunk) are
// numbered tile-fastest so the blocks resident at any moment work on
// neighbouring tiles of the same z range.
#include <algorithm>
#include <cmath>
#include <vector>

#include "axs_internal.cuh"

namespace axs {

int level_fill_ghosts(void *data, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g, int ncomp,
                      cudaStream_t st);
int level_copy_fab(void *lv, int32_t dtype, const LevelGeom &g, const axs_fab &f, int to_level, cudaStream_t st);

template <typename T> struct StageCoef {
    T kappa, hlam, R2;  // kappa, lambda/2, R^2 at one stage time
};

template <typename T> struct SweepArgs {
    int nx, ny, nz;
    int tiles_x, ntiles, zchunk;
    int64_t n_items;
    int64_t js, ks, cs;
    int ox;                     // x offset of the valid region in a padded row
    T wA, wB, wC;               // lap = wA*S1 + wB*S2 + wC*f0 (S1/S2: sums of +-1 / +-2 neighbours)
    StageCoef<T> ca, cb;        // sweep A: F1, F2; sweep B: F3, F4
    T h, h_half, h2_quarter, h2_half, h_sixth, h_third, h2_sixth;
    T *state;                   // sweep B output (4 comps, padded copies kept current)
    T *work;                    // sweep A output (8 comps); sweep B pointwise input (comps 4..7)
    unsigned *status;
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

template <typename T, int V>
__device__ __forceinline__ void store_with_copies(T *base, int64_t off, int x, int y, int nx, int ny, int64_t js,
                                                  const T *v)
{
    stv<T, V>(base + off, v);
    if (x < 4) stv<T, V>(base + off + nx, v);
    if (x >= nx - 4) stv<T, V>(base + off - nx, v);
    if (y < 2) stv<T, V>(base + off + (int64_t)ny * js, v);
    if (y >= ny - 2) stv<T, V>(base + off - (int64_t)ny * js, v);
}

template <typename T, int V, int TX, int TY, int NS, int MINB, int SWEEP>
__global__ void __launch_bounds__(SweepShape<T, V, TX, TY>::NT, MINB)
    rk4_sweep_kernel(const __grid_constant__ CUtensorMap tmap, const SweepArgs<T> a)
{
    using S = SweepShape<T, V, TX, TY>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *ring = reinterpret_cast<T *>(smem_raw);
    __shared__ uint64_t full[NS];
    __shared__ int abort_flag;

    const int tid = threadIdx.x;
    const int tx = tid % S::NTX, ty = tid / S::NTX;

    if (tid == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
        abort_flag = 0;
        prefetch_tensormap(&tmap);
    }
    __syncthreads();

    // ---- producer cursor (thread 0 only) ----
    int64_t p_item = blockIdx.x;
    int p_k = 0;
    int64_t q_issued = 0;
    auto issue_one = [&]() -> bool {
        if (p_item >= a.n_items) return false;
        const int tile = (int)(p_item % a.ntiles);
        const int chunk = (int)(p_item / a.ntiles);
        const int za = chunk * a.zchunk;
        const int len = min(a.zchunk, a.nz - za);
        int zp = (za - 2 + p_k) % a.nz;
        if (zp < 0) zp += a.nz;
        const int slot = (int)(q_issued % NS);
        mbar_arrive_expect_tx(&full[slot], S::SLOT_BYTES);
        // box x starts 4 columns left of the tile: padded column ox + x0 - 4 (16-byte aligned)
        tma_load_4d(ring + (size_t)slot * S::SLOT, &tmap, a.ox - 4 + (tile % a.tiles_x) * TX,
                    (tile / a.tiles_x) * TY, zp, 0, &full[slot]);
        ++q_issued;
        if (++p_k == len + 4) {
            p_k = 0;
            p_item += gridDim.x;
        }
        return true;
    };
    if (tid == 0) {
        for (int s = 0; s < NS; ++s)
            if (!issue_one()) break;
    }

    int64_t q_base = 0, q_waited = 0;
    bool aborted = false;
    const int xl = 4 + V * tx;  // tile-local column of this thread's first site
    const int yl = 2 + ty;
    for (int64_t item = blockIdx.x; item < a.n_items; item += gridDim.x) {
        const int tile = (int)(item % a.ntiles);
        const int chunk = (int)(item / a.ntiles);
        const int za = chunk * a.zchunk;
        const int len = min(a.zchunk, a.nz - za);
        const int x = (tile % a.tiles_x) * TX + V * tx;
        const int y = (tile / a.tiles_x) * TY + ty;
        const bool active = (x < a.nx) && (y < a.ny);
        // sweep B: the pointwise increments (G, P) of the next plane are loaded
        // one iteration ahead, so their latency hides behind a whole plane of work
        T gn[2][V], pn[2][V];
        if constexpr (SWEEP == 1) {
            if (active) {
                const int64_t off0 = (int64_t)(x + a.ox) + (int64_t)(y + 2) * a.js + (int64_t)za * a.ks;
                ldv_nc<T, V>(a.work + 4 * a.cs + off0, gn[0]);
                ldv_nc<T, V>(a.work + 5 * a.cs + off0, gn[1]);
                ldv_nc<T, V>(a.work + 6 * a.cs + off0, pn[0]);
                ldv_nc<T, V>(a.work + 7 * a.cs + off0, pn[1]);
            }
        }
        for (int m = 0; m < len; ++m) {
            const int z = za + m;
            const int64_t off = (int64_t)(x + a.ox) + (int64_t)(y + 2) * a.js + (int64_t)z * a.ks;

            T gq[2][V], pq[2][V];
            if constexpr (SWEEP == 1) {
#pragma unroll
                for (int i = 0; i < 2; ++i)
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        gq[i][v] = gn[i][v];
                        pq[i][v] = pn[i][v];
                    }
                if (active && m + 1 < len) {
                    ldv_nc<T, V>(a.work + 4 * a.cs + off + a.ks, gn[0]);
                    ldv_nc<T, V>(a.work + 5 * a.cs + off + a.ks, gn[1]);
                    ldv_nc<T, V>(a.work + 6 * a.cs + off + a.ks, pn[0]);
                    ldv_nc<T, V>(a.work + 7 * a.cs + off + a.ks, pn[1]);
                }
            }

            const int64_t need = q_base + m + 4;
            while (q_waited <= need) {
                const int slot = (int)(q_waited % NS);
                if (!mbar_wait_bounded(&full[slot], (uint32_t)((q_waited / NS) & 1))) {
                    atomicOr(a.status, kDevTimeout);
                    abort_flag = 1;
                }
                ++q_waited;
            }

            const T *sl[5];
#pragma unroll
            for (int d = 0; d < 5; ++d) sl[d] = ring + (size_t)((q_base + m + d) % NS) * S::SLOT;

            if (active) {
                T lap[4][V], ctr[4][V];
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const T *P0 = sl[2] + c * S::TILE;
                    T row[S::NROW * V], ym1[V], yp1[V], ym2[V], yp2[V], zm1[V], zp1[V], zm2[V], zp2[V];
#pragma unroll
                    for (int r = 0; r < S::NROW; ++r) ldv<T, V>(P0 + yl * S::BX + xl + (r - S::PRE) * V, row + r * V);
                    ldv<T, V>(P0 + (yl - 1) * S::BX + xl, ym1);
                    ldv<T, V>(P0 + (yl + 1) * S::BX + xl, yp1);
                    ldv<T, V>(P0 + (yl - 2) * S::BX + xl, ym2);
                    ldv<T, V>(P0 + (yl + 2) * S::BX + xl, yp2);
                    ldv<T, V>(sl[1] + c * S::TILE + yl * S::BX + xl, zm1);
                    ldv<T, V>(sl[3] + c * S::TILE + yl * S::BX + xl, zp1);
                    ldv<T, V>(sl[0] + c * S::TILE + yl * S::BX + xl, zm2);
                    ldv<T, V>(sl[4] + c * S::TILE + yl * S::BX + xl, zp2);
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        const int ci = S::PRE * V + v;
                        const T f0 = row[ci];
                        const T s1 = (row[ci - 1] + row[ci + 1]) + (ym1[v] + yp1[v]) + (zm1[v] + zp1[v]);
                        const T s2 = (row[ci - 2] + row[ci + 2]) + (ym2[v] + yp2[v]) + (zm2[v] + zp2[v]);
                        lap[c][v] = fma(a.wA, s1, fma(a.wB, s2, a.wC * f0));
                        ctr[c][v] = f0;
                    }
                }

                if constexpr (SWEEP == 0) {
                    T o[8][V];
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        const T p1 = ctr[0][v], p2 = ctr[1][v], q1 = ctr[2][v], q2 = ctr[3][v];
                        // F1 = F(t, psi_n)
                        const T k1 = fma(-a.ca.hlam, fma(p1, p1, p2 * p2) - a.ca.R2, a.ca.kappa);
                        const T f11 = fma(k1, p1, lap[0][v]);
                        const T f12 = fma(k1, p2, lap[1][v]);
                        // F2 = F(t + h/2, chi), chi = psi_n + h/2 Pi_n, lap(chi) = lap(psi) + h/2 lap(Pi)
                        const T c1 = fma(a.h_half, q1, p1), c2 = fma(a.h_half, q2, p2);
                        const T k2 = fma(-a.cb.hlam, fma(c1, c1, c2 * c2) - a.cb.R2, a.cb.kappa);
                        const T f21 = fma(k2, c1, fma(a.h_half, lap[2][v], lap[0][v]));
                        const T f22 = fma(k2, c2, fma(a.h_half, lap[3][v], lap[1][v]));
                        o[0][v] = fma(a.h2_quarter, f11, c1);                     // S3
                        o[1][v] = fma(a.h2_quarter, f12, c2);
                        o[2][v] = fma(a.h2_half, f21, fma(a.h, q1, p1));          // S4
                        o[3][v] = fma(a.h2_half, f22, fma(a.h, q2, p2));
                        o[4][v] = fma(T(-2), f21, f11);                          // G = F1 - 2 F2
                        o[5][v] = fma(T(-2), f22, f12);
                        o[6][v] = fma(a.h_third, f21, fma(a.h_sixth, f11, q1));  // P = Pi + h/6 F1 + h/3 F2
                        o[7][v] = fma(a.h_third, f22, fma(a.h_sixth, f12, q2));
                    }
#pragma unroll
                    for (int c = 0; c < 4; ++c)
                        store_with_copies<T, V>(a.work + c * a.cs, off, x, y, a.nx, a.ny, a.js, o[c]);
#pragma unroll
                    for (int c = 4; c < 8; ++c) stv<T, V>(a.work + c * a.cs + off, o[c]);
                } else {
                    T o[4][V];
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        const T s31 = ctr[0][v], s32 = ctr[1][v], s41 = ctr[2][v], s42 = ctr[3][v];
                        const T k3 = fma(-a.ca.hlam, fma(s31, s31, s32 * s32) - a.ca.R2, a.ca.kappa);
                        const T f31 = fma(k3, s31, lap[0][v]);
                        const T f32 = fma(k3, s32, lap[1][v]);
                        const T k4 = fma(-a.cb.hlam, fma(s41, s41, s42 * s42) - a.cb.R2, a.cb.kappa);
                        const T f41 = fma(k4, s41, lap[2][v]);
                        const T f42 = fma(k4, s42, lap[3][v]);
                        o[0][v] = fma(a.h2_sixth, gq[0][v] + f31, s41);
                        o[1][v] = fma(a.h2_sixth, gq[1][v] + f32, s42);
                        o[2][v] = fma(a.h_sixth, f41, fma(a.h_third, f31, pq[0][v]));
                        o[3][v] = fma(a.h_sixth, f42, fma(a.h_third, f32, pq[1][v]));
                    }
#pragma unroll
                    for (int c = 0; c < 4; ++c)
                        store_with_copies<T, V>(a.state + c * a.cs, off, x, y, a.nx, a.ny, a.js, o[c]);
                }
            }

            __syncthreads();  // everyone is done with the oldest plane of this window
            if (abort_flag) {
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
}

// ---------------------------------------------------------------- host side
int level_geom(int32_t dtype, int nx, int ny, int nz, LevelGeom &g)
{
    AXS_REQUIRE(dtype == AXS_F32 || dtype == AXS_F64, AXS_ERR_INVALID_ARGUMENT, "bad dtype %d", dtype);
    AXS_REQUIRE(nx > 0 && ny > 0 && nz > 0, AXS_ERR_INVALID_ARGUMENT, "empty level %dx%dx%d", nx, ny, nz);
    const int V = dtype == AXS_F64 ? 2 : 4;
    AXS_REQUIRE(nx % V == 0 && nx >= 4, AXS_ERR_UNSUPPORTED, "level nx must be a multiple of %d and >= 4 (got %d)", V,
                nx);
    AXS_REQUIRE(ny >= 2, AXS_ERR_UNSUPPORTED, "level ny must be >= 2 (got %d)", ny);
    const int line = 128 / (int)dtype_size(dtype);  // elements per 128-byte line
    g.ox = line;                                     // x = 0 starts a line; 4 periodic columns sit left of it
    g.oy = 2;
    g.js = ((int64_t)nx + g.ox + 4 + line - 1) / line * line;
    g.ks = g.js * (ny + 4);
    g.cs = g.ks * nz;
    return AXS_OK;
}

static int validate_level(const axs_level *lv, LevelGeom &g)
{
    AXS_REQUIRE(lv != nullptr, AXS_ERR_INVALID_ARGUMENT, "null level");
    AXS_REQUIRE(lv->state != nullptr && lv->work != nullptr, AXS_ERR_INVALID_ARGUMENT, "level state/work is null");
    int rc = level_geom(lv->dtype, lv->nx, lv->ny, lv->nz, g);
    if (rc) return rc;
    AXS_REQUIRE(lv->dx > 0.0, AXS_ERR_INVALID_ARGUMENT, "dx must be positive");
    AXS_REQUIRE(((uintptr_t)lv->state % 128) == 0 && ((uintptr_t)lv->work % 128) == 0, AXS_ERR_ALIGNMENT,
                "level buffers must be 128-byte aligned");
    return AXS_OK;
}

static unsigned *level_status_word(const axs_level *lv, const LevelGeom &g)
{
    const size_t es = dtype_size(lv->dtype);
    return reinterpret_cast<unsigned *>(static_cast<char *>(lv->work) + 8 * g.cs * es);
}

struct SweepRunArgs {
    const axs_level *lv;
    const LevelGeom *g;
    const axs_background *bg;
    double tau_i, t0, dt;
    int nsteps;
    int sweep_mask;
    cudaStream_t st;
};

// Pick the z-chunk length: balance the last wave against the 4 warm-up
// planes each chunk costs, and keep the SMs busy.
static void plan_chunks(int ntiles, int nz, int grid_cap, int &zchunk, int64_t &items, int &grid)
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

template <typename T, int V, int TX, int TY, int NS, int MINB> struct SweepConfig {
    using S = SweepShape<T, V, TX, TY>;
    static size_t smem() { return (size_t)NS * S::SLOT_BYTES; }

    static int prepare(int &blocks_per_sm)
    {
        static int cached = -1;
        if (cached < 0) {
            AXS_CUDA_CHECK(cudaFuncSetAttribute(rk4_sweep_kernel<T, V, TX, TY, NS, MINB, 0>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem()));
            AXS_CUDA_CHECK(cudaFuncSetAttribute(rk4_sweep_kernel<T, V, TX, TY, NS, MINB, 1>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem()));
            int b0 = 0, b1 = 0;
            AXS_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &b0, rk4_sweep_kernel<T, V, TX, TY, NS, MINB, 0>, S::NT, smem()));
            AXS_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &b1, rk4_sweep_kernel<T, V, TX, TY, NS, MINB, 1>, S::NT, smem()));
            cached = std::max(1, std::min(b0, b1));
        }
        blocks_per_sm = cached;
        return AXS_OK;
    }

    static int run(const SweepRunArgs &r)
    {
        const axs_level *lv = r.lv;
        const LevelGeom &g = *r.g;
        int bps = 0;
        int rc = prepare(bps);
        if (rc) return rc;
        const int sms = device_sm_count();
        AXS_REQUIRE(sms > 0, AXS_ERR_CUDA, "no CUDA device");
        const int tiles_x = (lv->nx + TX - 1) / TX, tiles_y = (lv->ny + TY - 1) / TY;
        SweepArgs<T> a{};
        a.nx = lv->nx;
        a.ny = lv->ny;
        a.nz = lv->nz;
        a.tiles_x = tiles_x;
        a.ntiles = tiles_x * tiles_y;
        int grid = 0;
        plan_chunks(a.ntiles, lv->nz, bps * sms, a.zchunk, a.n_items, grid);
        a.js = g.js;
        a.ks = g.ks;
        a.cs = g.cs;
        a.ox = g.ox;
        const double inv_dx2 = 1.0 / (lv->dx * lv->dx);
        a.wA = T((4.0 / 3.0) * inv_dx2);
        a.wB = T((-1.0 / 12.0) * inv_dx2);
        a.wC = T(-7.5 * inv_dx2);
        const double h = r.dt;
        a.h = T(h);
        a.h_half = T(0.5 * h);
        a.h2_quarter = T(0.25 * h * h);
        a.h2_half = T(0.5 * h * h);
        a.h_sixth = T(h / 6.0);
        a.h_third = T(h / 3.0);
        a.h2_sixth = T(h * h / 6.0);
        a.state = static_cast<T *>(lv->state);
        a.work = static_cast<T *>(lv->work);
        a.status = level_status_word(lv, g);

        const size_t es = sizeof(T);
        CUtensorMap map_state, map_work;
        rc = make_tensor_map_4d(&map_state, lv->state, lv->dtype, g.js, lv->ny + 4, lv->nz, 4, g.js * es, g.ks * es,
                                g.cs * es, S::BX, S::BY, 1, 4);
        if (rc) return rc;
        rc = make_tensor_map_4d(&map_work, lv->work, lv->dtype, g.js, lv->ny + 4, lv->nz, 4, g.js * es, g.ks * es,
                                g.cs * es, S::BX, S::BY, 1, 4);
        if (rc) return rc;

        auto coef = [&](double tau) {
            axs_rhs_coeffs c;
            rhs_coeffs(*r.bg, tau, c);
            return StageCoef<T>{T(c.kappa), T(0.5 * c.lambda), T(c.R2)};
        };
        for (int s = 0; s < r.nsteps; ++s) {
            const double t = r.t0 + s * r.dt;
            if (r.sweep_mask & 1) {
                SweepArgs<T> aa = a;
                aa.ca = coef(r.tau_i + t);
                aa.cb = coef(r.tau_i + t + 0.5 * r.dt);
                rk4_sweep_kernel<T, V, TX, TY, NS, MINB, 0><<<grid, S::NT, smem(), r.st>>>(map_state, aa);
                rc = launch_status("rk4 sweep A");
                if (rc) return rc;
            }
            if (r.sweep_mask & 2) {
                SweepArgs<T> ab = a;
                ab.ca = coef(r.tau_i + t + 0.5 * r.dt);
                ab.cb = coef(r.tau_i + t + r.dt);
                rk4_sweep_kernel<T, V, TX, TY, NS, MINB, 1><<<grid, S::NT, smem(), r.st>>>(map_work, ab);
                rc = launch_status("rk4 sweep B");
                if (rc) return rc;
            }
        }
        return AXS_OK;
    }
};

// Tile configurations (vector width, tile, ring depth, expected blocks/SM).
// Entry 0 of each table is the default (tile_config = 0).
struct TileConfigEntry {
    const char *name;
    int (*run)(const SweepRunArgs &);
};

static const TileConfigEntry kF32Configs[] = {
    {"f32 v2 64x8 ring8", &SweepConfig<float, 2, 64, 8, 8, 2>::run},
    {"f32 v2 32x16 ring8", &SweepConfig<float, 2, 32, 16, 8, 2>::run},
    {"f32 v4 32x16 ring8", &SweepConfig<float, 4, 32, 16, 8, 2>::run},
    {"f32 v2 32x8 ring8", &SweepConfig<float, 2, 32, 8, 8, 3>::run},
    {"f32 v1 32x8 ring8", &SweepConfig<float, 1, 32, 8, 8, 3>::run},
    {"f32 v2 64x8 ring10", &SweepConfig<float, 2, 64, 8, 10, 1>::run},
    {"f32 v4 64x16 ring6", &SweepConfig<float, 4, 64, 16, 6, 1>::run},
    {"f32 v2 32x16 ring6", &SweepConfig<float, 2, 32, 16, 6, 2>::run},
    {"f32 v1 32x16 ring7", &SweepConfig<float, 1, 32, 16, 7, 2>::run},
};
static const TileConfigEntry kF64Configs[] = {
    {"f64 v1 32x8 ring6", &SweepConfig<double, 1, 32, 8, 6, 2>::run},
    {"f64 v2 32x8 ring6", &SweepConfig<double, 2, 32, 8, 6, 2>::run},
    {"f64 v2 32x16 ring6", &SweepConfig<double, 2, 32, 16, 6, 1>::run},
    {"f64 v1 32x4 ring7", &SweepConfig<double, 1, 32, 4, 7, 3>::run},
};

static int config_count(int32_t dtype)
{
    return dtype == AXS_F64 ? (int)(sizeof(kF64Configs) / sizeof(kF64Configs[0]))
                            : (int)(sizeof(kF32Configs) / sizeof(kF32Configs[0]));
}

static const TileConfigEntry *config_for(int32_t dtype, int32_t id)
{
    const TileConfigEntry *tab = dtype == AXS_F64 ? kF64Configs : kF32Configs;
    if (id < 0 || id > config_count(dtype)) return nullptr;
    return &tab[id == 0 ? 0 : id - 1];
}

static int run_sweeps(const axs_level *lv, const LevelGeom &g, const axs_background *bg, double tau_i, double t0,
                      double dt, int nsteps, int mask, cudaStream_t st)
{
    const TileConfigEntry *cfg = config_for(lv->dtype, lv->tile_config);
    AXS_REQUIRE(cfg != nullptr, AXS_ERR_INVALID_ARGUMENT, "tile_config %d out of range (0..%d)", lv->tile_config,
                config_count(lv->dtype));
    SweepRunArgs r{lv, &g, bg, tau_i, t0, dt, nsteps, mask, st};
    return cfg->run(r);
}

}  // namespace axs

using namespace axs;

extern "C" {

int axs_level_layout_for(int32_t dtype, int32_t nx, int32_t ny, int32_t nz, axs_level_layout *out)
{
    AXS_REQUIRE(out != nullptr, AXS_ERR_INVALID_ARGUMENT, "null output");
    LevelGeom g;
    int rc = level_geom(dtype, nx, ny, nz, g);
    if (rc) return rc;
    const int64_t es = (int64_t)dtype_size(dtype);
    out->jstride = g.js;
    out->kstride = g.ks;
    out->cstride = g.cs;
    out->x_offset = g.ox;
    out->y_offset = g.oy;
    out->state_bytes = 4 * g.cs * es;
    out->work_bytes = 8 * g.cs * es + 256;
    return AXS_OK;
}

int axs_level_tile_config_count(int32_t dtype)
{
    if (dtype != AXS_F32 && dtype != AXS_F64) return 0;
    return config_count(dtype);
}

const char *axs_level_tile_config_name(int32_t dtype, int32_t id)
{
    if (dtype != AXS_F32 && dtype != AXS_F64) return nullptr;
    const TileConfigEntry *c = config_for(dtype, id);
    return c ? c->name : nullptr;
}

int axs_level_fill_ghosts(const axs_level *lv, void *stream)
{
    LevelGeom g;
    int rc = validate_level(lv, g);
    if (rc) return rc;
    return level_fill_ghosts(lv->state, lv->dtype, lv->nx, lv->ny, lv->nz, g, 4, (cudaStream_t)stream);
}

int axs_level_import_fab(const axs_level *lv, const axs_fab *src, void *stream)
{
    LevelGeom g;
    int rc = validate_level(lv, g);
    if (rc) return rc;
    if ((rc = validate_fab(src, "src", 4, 0))) return rc;
    AXS_REQUIRE(src->dtype == lv->dtype && src->nx == lv->nx && src->ny == lv->ny && src->nz == lv->nz,
                AXS_ERR_INVALID_ARGUMENT, "FAB and level differ in dtype or extent");
    rc = level_copy_fab(lv->state, lv->dtype, g, *src, 1, (cudaStream_t)stream);
    if (rc) return rc;
    return level_fill_ghosts(lv->state, lv->dtype, lv->nx, lv->ny, lv->nz, g, 4, (cudaStream_t)stream);
}

int axs_level_export_fab(const axs_level *lv, const axs_fab *dst, void *stream)
{
    LevelGeom g;
    int rc = validate_level(lv, g);
    if (rc) return rc;
    if ((rc = validate_fab(dst, "dst", 4, 0))) return rc;
    AXS_REQUIRE(dst->dtype == lv->dtype && dst->nx == lv->nx && dst->ny == lv->ny && dst->nz == lv->nz,
                AXS_ERR_INVALID_ARGUMENT, "FAB and level differ in dtype or extent");
    return level_copy_fab(lv->state, lv->dtype, g, *dst, 0, (cudaStream_t)stream);
}

int axs_level_rk4_advance(const axs_level *lv, const axs_background *bg, double tau_i, double t0, double dt,
                          int32_t nsteps, void *stream)
{
    LevelGeom g;
    int rc = validate_level(lv, g);
    if (rc) return rc;
    AXS_REQUIRE(bg != nullptr, AXS_ERR_INVALID_ARGUMENT, "null background");
    AXS_REQUIRE(nsteps >= 0, AXS_ERR_INVALID_ARGUMENT, "negative step count");
    AXS_REQUIRE(std::isfinite(dt) && dt > 0.0, AXS_ERR_INVALID_ARGUMENT, "dt must be positive and finite");
    if (bg->kind == AXS_BG_EXPANDING) {
        AXS_REQUIRE(bg->a_inv > 1.0, AXS_ERR_INVALID_ARGUMENT, "a_inv must exceed 1");
        AXS_REQUIRE(tau_i + t0 > 0.0, AXS_ERR_INVALID_ARGUMENT, "conformal time must stay positive");
    }
    if (nsteps == 0) return AXS_OK;
    return run_sweeps(lv, g, bg, tau_i, t0, dt, nsteps, 3, (cudaStream_t)stream);
}

int axs_level_rk4_sweep(const axs_level *lv, const axs_background *bg, double tau_i, double t, double dt,
                        int32_t sweep, void *stream)
{
    LevelGeom g;
    int rc = validate_level(lv, g);
    if (rc) return rc;
    AXS_REQUIRE(bg != nullptr, AXS_ERR_INVALID_ARGUMENT, "null background");
    AXS_REQUIRE(sweep == 0 || sweep == 1, AXS_ERR_INVALID_ARGUMENT, "sweep must be 0 (A) or 1 (B)");
    AXS_REQUIRE(std::isfinite(dt) && dt > 0.0, AXS_ERR_INVALID_ARGUMENT, "dt must be positive and finite");
    return run_sweeps(lv, g, bg, tau_i, t, dt, 1, sweep == 0 ? 1 : 2, (cudaStream_t)stream);
}

int axs_level_device_status(const axs_level *lv, void *stream)
{
    LevelGeom g;
    int rc = validate_level(lv, g);
    if (rc) return rc;
    unsigned host = 0;
    unsigned *dev = level_status_word(lv, g);
    AXS_CUDA_CHECK(cudaMemcpyAsync(&host, dev, sizeof(unsigned), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    AXS_CUDA_CHECK(cudaStreamSynchronize((cudaStream_t)stream));
    if (host) {
        AXS_CUDA_CHECK(cudaMemsetAsync(dev, 0, sizeof(unsigned), (cudaStream_t)stream));
        AXS_CUDA_CHECK(cudaStreamSynchronize((cudaStream_t)stream));
        set_error("a device-side wait timed out (status word 0x%x)", host);
        return AXS_ERR_DEVICE_TIMEOUT;
    }
    return AXS_OK;
}

}  // extern "C"
