// One-pass fused RK4 step of a periodic level (FP32).
//
// The two sweeps of a step (rk4_level.cu) move 28 words per site: sweep A
// writes the stage increments (d3, d4, E, Q) to HBM and sweep B reads them
// back. This kernel keeps them on chip. A CTA owns a TX x TY tile of the xy
// plane over a chunk of z planes and marches in z. Per plane it
//   - runs sweep A on the tile plus a 2-cell halo (the A region) from a TMA
//     ring of (psi, Pi) planes with a 4-cell halo,
//   - keeps d3, d4 (A region, 6 planes) and E, Q (tile, 4 planes) in shared
//     memory,
//   - runs sweep B two planes behind on the tile and writes psi, Pi of the
//     step's end to the other state buffer.
// level_pad_kernel then writes the periodic copies of that buffer's padding
// (8 columns, 2 rows and their corners): kept out of the step's loop, whose
// code the copy branches slowed by 8 % although few tiles take them.
// Reading one buffer and writing the other makes the tiles independent (no
// tile reads what another writes), so the CTAs need no synchronisation with
// each other; the level's work buffer serves as the second state buffer and
// steps alternate between the two. A step moves 8 words per site (psi, Pi in
// and out) plus the halo rows the L2 does not catch, against 28 for the two
// sweeps; in return sweep A runs on (TX+4)(TY+4) sites per TX*TY.
//
// The per-site arithmetic is the two sweeps' own (lap_pair, stage_a,
// stage_b), so both paths give the same bits.
//
// Halo: the box is (TX+16) x (TY+8) x 1 plane x 4 components, starting 8
// columns and 4 rows before the tile. In x the level's 8 padding columns hold
// the periodic copies; reading 8 columns (not the 4 the stencil needs) on
// either side makes two box rows a whole number of 128-byte lines, so each
// piece of a split box below lands 128-byte aligned. In y the padding holds 2
// rows: tiles in the first or last row of tiles load their 4 components as
// three pieces each (2 rows from the wrapped edge, the TY+4 rows through the
// padding, 2 more wrapped rows). z wraps by plane index. The corners of the
// padding are read here: the periodic stores write them.
#pragma once

#include "rk4_ops.cuh"

namespace axs {

template <int TX_, int TY_, int NS_, int THREADS_ = 512, bool COMP_ = false> struct LevelFusedShape {
    using T = float;
    static constexpr bool COMP = COMP_;  // the compensated FP32 step (stage_a in rk4_ops.cuh)
    static constexpr int V = 2, TX = TX_, TY = TY_, NS = NS_;
    // sweep A units run on the first NA threads and sweep B units on the last NB:
    // with 640 threads no thread runs both, so sweep B of one plane overlaps sweep
    // A of the next; with 512 some threads run both every plane
    static constexpr int THREADS = THREADS_;
    static constexpr int BX = TX + 16, BY = TY + 8;  // TMA box: the A region, its stencil halo, alignment columns
    static constexpr int AX = TX + 4, AY = TY + 4;   // A region
    static constexpr int RING = 4 * BX * BY, SWIN = 4 * AX * AY, EQW = 4 * TX * TY;
    // d3, d4 slots (sweep B reads 5 planes; one more so that sweep A of the next
    // plane never overwrites a slot a slower thread still reads) and E, Q slots
    // (written two planes before sweep B reads them, plus the same margin)
    static constexpr int NSW = 6, NEQ = 4;
    static_assert(NS >= 6 && NS <= 10 && NEQ == 4, "slot arithmetic below (wrap by one subtraction, E/Q by xor)");
    static constexpr int NA = AX * AY / V;  // sweep A units (V sites each)
    static constexpr int NB = TX * TY / V;  // sweep B units, one per thread of the last NB threads
    static constexpr size_t SMEM = sizeof(T) * ((size_t)NS * RING + NSW * (size_t)SWIN + NEQ * (size_t)EQW);
    static constexpr uint32_t SLOT_BYTES = RING * sizeof(T);
    static_assert(NA <= THREADS && NB <= THREADS, "at most one unit of each sweep per thread");
    static_assert(THREADS % 32 == 0 && THREADS <= 1024, "whole warps");
    static_assert((2 * BX * sizeof(T)) % 128 == 0 && ((TY + 6) * BX * sizeof(T)) % 128 == 0,
                  "the pieces of a split box land 128-byte aligned");
    static_assert((BX * sizeof(T)) % 16 == 0, "TMA box rows of whole 16-byte units");
    static_assert((RING * sizeof(T)) % 128 == 0 && (BX * BY * sizeof(T)) % 128 == 0, "ring slots and components");
    static_assert(AX / V > 32 / V, "the A region is wider than one bank row");
    static_assert(BX <= 256 && BY <= 256, "TMA box extent limit");
    static_assert(SMEM + 1024 <= 227 * 1024, "shared memory");
};

// Shared-memory accesses by 32-bit shared address plus a compile-time byte
// offset, one instruction each.
template <int OFF> __device__ __forceinline__ float2 lds2(uint32_t addr)
{
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2+%3];" : "=f"(v.x), "=f"(v.y) : "r"(addr), "n"(OFF));
    return v;
}
template <int OFF> __device__ __forceinline__ void sts2(uint32_t addr, float x, float y)
{
    asm volatile("st.shared.v2.f32 [%0+%1], {%2, %3};" ::"r"(addr), "n"(OFF), "f"(x), "f"(y) : "memory");
}

// Laplacian and centre of two sites of one component: p[d] = shared address of
// the first site in planes z-2 .. z+2, RB the row length in bytes, CO the
// component's byte offset. The arithmetic is lap_pair's, as in every FP32 sweep.
template <int RB, int CO, bool COMP>
__device__ __forceinline__ void star_pair_sh(const SweepArgs<float> &a, const uint32_t (&p)[5], float (&lap)[2],
                                             float (&ctr)[2])
{
    const float2 a0 = lds2<CO - 8>(p[2]), a1 = lds2<CO>(p[2]), a2 = lds2<CO + 8>(p[2]);
    const float r[6] = {a0.x, a0.y, a1.x, a1.y, a2.x, a2.y};
    lap_pair<COMP>(a, r, lds2<CO - RB>(p[2]), lds2<CO + RB>(p[2]), lds2<CO - 2 * RB>(p[2]), lds2<CO + 2 * RB>(p[2]),
                   lds2<CO>(p[1]), lds2<CO>(p[3]), lds2<CO>(p[0]), lds2<CO>(p[4]), lap[0], lap[1]);
    ctr[0] = a1.x;
    ctr[1] = a1.y;
}

// the same for the four components, CS bytes apart
template <int RB, int CS, bool COMP>
__device__ __forceinline__ void star4_sh(const SweepArgs<float> &a, const uint32_t (&p)[5], float (&lap)[4][2],
                                         float (&ctr)[4][2])
{
    star_pair_sh<RB, 0 * CS, COMP>(a, p, lap[0], ctr[0]);
    star_pair_sh<RB, 1 * CS, COMP>(a, p, lap[1], ctr[1]);
    star_pair_sh<RB, 2 * CS, COMP>(a, p, lap[2], ctr[2]);
    star_pair_sh<RB, 3 * CS, COMP>(a, p, lap[3], ctr[3]);
}

// The three tensor maps over one state buffer: the whole box (interior tile
// rows), one component of TY + 4 rows, one component of 2 rows.
struct LevelFusedMaps {
    CUtensorMap full, mid, rows2;
};

// A work item of the fused step: a TX x TY tile over a chunk of z planes of
// one periodic box, with the box's geometry and the three tensor maps of the
// buffer the step reads.
struct FusedItem {
    int x0, y0, z0, len;
    int nx, ny, nz;
    int64_t js, ks, base;  // base: element offset of the box in every component plane
    const CUtensorMap *full, *mid, *rows2;
};

// A block's walk over its work items (the producer thread and the consumers
// each keep one).
struct FusedCursor {
    int64_t pos, end;
};

// Work-item sources of the fused step: begin / valid / item / next.
// One periodic level in (tile, z-chunk) items, taken by blocks in turn;
// geometry from the launch parameters, nx a multiple of TX.
struct FusedLevel {
    static constexpr bool kPartialX = false;
    static constexpr bool kMapsInTable = false;  // maps by value in the launch parameters
    __device__ __forceinline__ static FusedCursor begin(const SweepArgs<float> &a) { return {blockIdx.x, a.n_items}; }
    __device__ __forceinline__ static bool valid(const FusedCursor &c) { return c.pos < c.end; }
    __device__ __forceinline__ static void next(FusedCursor &c, int) { c.pos += gridDim.x; }
    template <int TX, int TY>
    __device__ __forceinline__ static FusedItem item(const SweepArgs<float> &a, const LevelFusedMaps &m,
                                                     const FusedCursor &c)
    {
        const int tile = (int)(c.pos % a.ntiles);
        const int z0 = (int)(c.pos / a.ntiles) * a.zchunk;
        return FusedItem{(tile % a.tiles_x) * TX, (tile / a.tiles_x) * TY, z0, min(a.zchunk, a.nz - z0), a.nx, a.ny,
                         a.nz, a.js, a.ks, 0, &m.full, &m.mid, &m.rows2};
    }
};
// The boxes of an ensemble: the item list and box descriptors of a box table,
// and per box six tensor maps in the table (full, mid, rows2 over each of the
// two state buffers; map_sel picks the buffer read). ny is a multiple of TY.
// The last tile column of a box whose width is not a multiple of TX runs past
// the box: its stores are masked. Its sweep A sites up to nx + 1 read the
// padding copies (8 columns) and feed the last valid sites; the ones further
// right read zero-filled or unused columns and feed only masked sites.
struct FusedBoxes {
    static constexpr bool kPartialX = true;
    static constexpr bool kMapsInTable = true;  // written by a host copy: acquired before use
    __device__ __forceinline__ static FusedCursor begin(const SweepArgs<float> &a) { return {blockIdx.x, a.n_items}; }
    __device__ __forceinline__ static bool valid(const FusedCursor &c) { return c.pos < c.end; }
    __device__ __forceinline__ static void next(FusedCursor &c, int) { c.pos += gridDim.x; }
    template <int TX, int TY>
    __device__ __forceinline__ static FusedItem item(const SweepArgs<float> &a, const LevelFusedMaps &,
                                                     const FusedCursor &c)
    {
        const uint32_t e = __ldg(a.items + c.pos);
        const EnsBoxDesc &d = a.boxes[e >> kEnsItemBits];
        const int local = (int)(e & ((1u << kEnsItemBits) - 1));
        const int tile = local % d.ntiles;
        const int z0 = (local / d.ntiles) * d.zchunk;
        const CUtensorMap *m = a.maps + 3 * (2 * d.map_box + a.map_sel);
        return FusedItem{(tile % d.tiles_x) * TX, (tile / d.tiles_x) * TY, z0, min(d.zchunk, d.nz - z0), d.nx, d.ny,
                         d.nz, d.js, d.ks, d.base, m, m + 1, m + 2};
    }
};

template <class S, class Src = FusedLevel>
__global__ void __launch_bounds__(S::THREADS, 1)
    level_fused_kernel(const __grid_constant__ LevelFusedMaps maps, const SweepArgs<float> a)
{
    using T = float;
    constexpr int V = S::V, TX = S::TX, TY = S::TY, NS = S::NS, BX = S::BX, BY = S::BY, AX = S::AX, AY = S::AY;
    extern __shared__ __align__(128) unsigned char lf_smem[];
    T *ring = reinterpret_cast<T *>(lf_smem);
    T *swin = ring + (size_t)NS * S::RING;
    T *eqw = swin + (size_t)S::NSW * S::SWIN;
    __shared__ uint64_t full[NS];
    const int tid = threadIdx.x;
    constexpr int oy = 2;  // padded row of y = 0 in the level layout

    if (tid == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
        prefetch_tensormap(&maps.full);
        prefetch_tensormap(&maps.mid);
        prefetch_tensormap(&maps.rows2);
    }
    __syncthreads();

    // ---- producer cursor (thread 0 only): planes z0 - 4 .. z0 + len + 3 of each item
    FusedCursor p_cur = Src::begin(a);
    int p_k = 0;
    FusedItem p{};
    bool p_edge = false;
    auto p_start = [&]() {
        if (!Src::valid(p_cur)) return;
        p = Src::template item<TX, TY>(a, maps, p_cur);
        p_edge = p.y0 == 0 || p.y0 + TY == p.ny;  // rows y0 - 4, y0 - 3 or y0 + TY + 2, + 3 lie past the padding
        if constexpr (Src::kMapsInTable) {
            fence_tensormap_acquire(p.full);
            fence_tensormap_acquire(p.mid);
            fence_tensormap_acquire(p.rows2);
        }
    };
    int64_t q_issued = 0;
    int p_slot = 0;  // ring slot of plane q_issued
    auto issue_one = [&]() -> bool {
        if (!Src::valid(p_cur)) return false;
        int zp = (p.z0 - 4 + p_k) % p.nz;
        if (zp < 0) zp += p.nz;
        const int slot = p_slot;
        if (++p_slot == NS) p_slot = 0;
        T *dst = ring + (size_t)slot * S::RING;
        mbar_arrive_expect_tx(&full[slot], S::SLOT_BYTES);
        const int xc = a.ox - 8 + p.x0;  // padded column of the box's first column (16-byte aligned)
        if (!p_edge) {
            tma_load_4d(dst, p.full, xc, p.y0 - 4 + oy, zp, 0, &full[slot]);
        } else {
            const int rt = ((p.y0 - 4) % p.ny + p.ny) % p.ny + oy;  // rows y0 - 4, y0 - 3 (wrapped)
            const int rb = (p.y0 + TY + 2) % p.ny + oy;            // rows y0 + TY + 2, + 3 (wrapped)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                T *dc = dst + (size_t)c * BX * BY;
                tma_load_4d(dc, p.rows2, xc, rt, zp, c, &full[slot]);
                tma_load_4d(dc + 2 * BX, p.mid, xc, p.y0 - 2 + oy, zp, c, &full[slot]);
                tma_load_4d(dc + (TY + 6) * BX, p.rows2, xc, rb, zp, c, &full[slot]);
            }
        }
        ++q_issued;
        if (++p_k == p.len + 8) {
            p_k = 0;
            Src::next(p_cur, p.len);
            p_start();
        }
        return true;
    };
    if (tid == 0) {
        p_start();
        for (int s = 0; s < NS; ++s)
            if (!issue_one()) break;
    }

    // sweep B unit of this thread (bt < 0: none), tile-local sites (bxl, byl) .. (bxl + V - 1, byl)
    const int bt = tid - (S::THREADS - S::NB);
    const bool has_b = bt >= 0;
    const int bxl = has_b ? V * (bt % (TX / V)) : 0, byl = has_b ? bt / (TX / V) : 0;
    // sweep A unit of this thread: units of the A region's first 32 / V columns row by
    // row (a warp covers whole 128-byte bank rows: conflict-free), then the others
    const bool has_a = tid < S::NA;
    int alx = 0, aly = 0;  // A-region-local first site
    {
        constexpr int PR = AX / V, MAIN = 32 / V, EDGE = PR - MAIN;
        const int u = tid;
        const int row = u < MAIN * AY ? u / MAIN : (u - MAIN * AY) / EDGE;
        const int col = u < MAIN * AY ? u % MAIN : MAIN + (u - MAIN * AY) % EDGE;
        alx = V * col;
        aly = row;
    }
    const int atx = alx - 2, aty = aly - 2;  // tile-local (V sites lie all inside or all outside the tile)
    const bool a_in_tile = atx >= 0 && atx < TX && aty >= 0 && aty < TY;
    // shared addresses of the three regions and this thread's byte offsets in them
    const uint32_t ring_sh = smem_addr(ring), swin_sh = smem_addr(swin), eqw_sh = smem_addr(eqw);
    const uint32_t a_at = 4u * (uint32_t)((aly + 2) * BX + (alx + 6));      // A site in the ring box
    const uint32_t a_so = 4u * (uint32_t)(aly * AX + alx);                  // A site in the d3, d4 window
    const uint32_t a_eo = 4u * (uint32_t)(a_in_tile ? aty * TX + atx : 0);  // A site in the E, Q window
    const uint32_t b_ro = 4u * (uint32_t)((byl + 4) * BX + (bxl + 8));     // B site in the ring box
    const uint32_t b_so = 4u * (uint32_t)((byl + 2) * AX + (bxl + 2));     // B site in the d3, d4 window
    const uint32_t b_eo = 4u * (uint32_t)(byl * TX + bxl);                 // B site in the E, Q window

    // Ring slots, their mbarrier phases and the window slots advance by one per
    // plane: rotating small counters (a modulo by the slot count per plane and
    // thread is a real cost in this issue-bound loop).
    int r0 = 0;                   // ring slot of plane q_base + i (the oldest plane sweep A reads)
    int w_slot = 0, w_phase = 0;  // the next plane to wait for: its slot and mbarrier parity
    int s0 = 0, e0 = 0;           // d3, d4 slot and E, Q slot of sweep A's plane
    int64_t q_waited = 0;
    bool aborted = false;
    for (FusedCursor cur = Src::begin(a); Src::valid(cur);) {
        const FusedItem w = Src::template item<TX, TY>(a, maps, cur);
        const int z0 = w.z0, len = w.len;
        // this thread's sweep B sites: element offset of their row at z = 0, and
        // whether they lie in the box
        const int64_t b_row = w.base + (int64_t)(w.x0 + bxl + a.ox) + (int64_t)(w.y0 + byl + oy) * w.js;
        const bool b_in = !Src::kPartialX || w.x0 + bxl < w.nx;
        // iteration i: sweep A at plane za = z0 - 2 + i (ring planes q_base + i .. + 4),
        // sweep B at zb = za - 2 = z0 - 4 + i for i >= 4
        for (int i = 0; i < len + 4; ++i) {
            // planes up to q_base + i + 4 must have landed: the first iteration of an
            // item waits for five, every later one for one more
            bool late = false;  // this thread's wait expired
            for (int need = i == 0 ? 5 : 1; need > 0; --need) {
                if (!mbar_wait_bounded(&full[w_slot], (uint32_t)w_phase, a.wait_polls)) {
                    atomicOr(a.status, kDevTimeout);
                    late = true;
                }
                ++q_waited;
                if (++w_slot == NS) {
                    w_slot = 0;
                    w_phase ^= 1;
                }
            }
            uint32_t pl[5];  // shared addresses of ring planes q_base + i .. + 4
#pragma unroll
            for (int d = 0; d < 5; ++d) {
                const int sd = r0 + d < NS ? r0 + d : r0 + d - NS;
                pl[d] = ring_sh + (uint32_t)sd * (uint32_t)(S::RING * 4);
            }
            if (has_a) {
                uint32_t pa[5];
#pragma unroll
                for (int d = 0; d < 5; ++d) pa[d] = pl[d] + a_at;
                T lap[4][V], ctr[4][V];
                star4_sh<BX * 4, BX * BY * 4, S::COMP>(a, pa, lap, ctr);
                T o[8][V];
                stage_a<T, V, S::COMP>(a, lap, ctr, o);
                const uint32_t sz = swin_sh + (uint32_t)s0 * (uint32_t)(S::SWIN * 4) + a_so;  // d3, d4 of plane za
                sts2<0 * AX * AY * 4>(sz, o[0][0], o[0][1]);
                sts2<1 * AX * AY * 4>(sz, o[1][0], o[1][1]);
                sts2<2 * AX * AY * 4>(sz, o[2][0], o[2][1]);
                sts2<3 * AX * AY * 4>(sz, o[3][0], o[3][1]);
                if (a_in_tile) {
                    const uint32_t ez = eqw_sh + (uint32_t)e0 * (uint32_t)(S::EQW * 4) + a_eo;  // E, Q of plane za
                    sts2<0 * TX * TY * 4>(ez, o[4][0], o[4][1]);
                    sts2<1 * TX * TY * 4>(ez, o[5][0], o[5][1]);
                    sts2<2 * TX * TY * 4>(ez, o[6][0], o[6][1]);
                    sts2<3 * TX * TY * 4>(ez, o[7][0], o[7][1]);
                }
            }
            // sweep B's psi_n, Pi_n at plane zb: ring plane q_base + i, refilled after the barrier
            float2 pn[4];
            if (has_b && i >= 4) {
                const uint32_t r0p = pl[0] + b_ro;
                pn[0] = lds2<0 * BX * BY * 4>(r0p);
                pn[1] = lds2<1 * BX * BY * 4>(r0p);
                pn[2] = lds2<2 * BX * BY * 4>(r0p);
                pn[3] = lds2<3 * BX * BY * 4>(r0p);
            }
            // d3, d4, E, Q of plane za are in place; ring plane q_base + i is read no
            // more. The barrier also ORs the threads' expired waits: a thread whose
            // wait expired ran its sweeps on a slot that may still be landing, and
            // the block drops those results here, before any global store (one
            // block-wide flag in shared memory, read three times a plane, cost
            // 1.4 % of the step).
            if (__syncthreads_or(late)) {
                aborted = true;
                break;
            }
            if (tid == 0) {
                // the oldest plane still needed: q_base + i + 1, or the next item's first
                const int64_t next_needed = q_waited - 4 + (i + 1 < len + 4 ? 0 : 4);
                fence_proxy_async_smem();
                while (q_issued < next_needed + NS && issue_one()) {
                }
            }
            if (has_b && i >= 4) {
                const int zb = z0 - 4 + i;
                const int b0 = s0 + 2 < S::NSW ? s0 + 2 : s0 + 2 - S::NSW;  // slot of plane za - 4 = zb - 2
                uint32_t sp[5];
#pragma unroll
                for (int d = 0; d < 5; ++d) {
                    const int sd = b0 + d < S::NSW ? b0 + d : b0 + d - S::NSW;
                    sp[d] = swin_sh + (uint32_t)sd * (uint32_t)(S::SWIN * 4) + b_so;
                }
                const uint32_t ez = eqw_sh + (uint32_t)(e0 ^ 2) * (uint32_t)(S::EQW * 4) + b_eo;  // E, Q of plane zb
                T lap[4][V], ctr[4][V], o[4][V], pq[8][V];
                star4_sh<AX * 4, AX * AY * 4, S::COMP>(a, sp, lap, ctr);
                const float2 e[4] = {lds2<0 * TX * TY * 4>(ez), lds2<1 * TX * TY * 4>(ez), lds2<2 * TX * TY * 4>(ez),
                                     lds2<3 * TX * TY * 4>(ez)};
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    pq[c][0] = e[c].x;
                    pq[c][1] = e[c].y;
                    pq[4 + c][0] = pn[c].x;
                    pq[4 + c][1] = pn[c].y;
                }
                stage_b<T, V, decltype(pq), S::COMP>(a, lap, ctr, pq, o);
                const int64_t off = b_row + (int64_t)zb * w.ks;
                if (b_in) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) stv<T, V>(a.out[c] + off, o[c]);
                }
            }
            if (++r0 == NS) r0 = 0;
            if (++s0 == S::NSW) s0 = 0;
            e0 = (e0 + 1) & (S::NEQ - 1);
        }
        if (aborted) break;
        // the next item's window starts 4 planes past this item's last window start + 1
        r0 += 4;
        if (r0 >= NS) r0 -= NS;
        Src::next(cur, len);
    }
    // A wait expired: make sure no bulk copy is still landing in shared memory
    // before the block exits (bounded as well).
    if (aborted && tid == 0) {
        for (int64_t q = q_waited; q < q_issued; ++q) mbar_wait_bounded(&full[q % NS], (uint32_t)((q / NS) & 1), 1u << 20);
    }
}

// The periodic padding of one level-layout buffer (4 components): columns
// x = -8 .. -1 and nx .. nx+7 of rows y = -2 .. ny+1, and rows y = -2, -1, ny,
// ny+1 of columns 0 .. nx-1, each a copy of the valid cell it wraps to. Grid
// rows are planes (z + nz c); within a plane, consecutive threads take
// consecutive elements of a padding row, and each thread copies kPadUnroll
// elements a grid-row stride apart, all loads before the stores (sources are
// valid cells, destinations padding: no copy reads another's destination).
constexpr int kPadUnroll = 4;
template <typename T>
__device__ __forceinline__ void pad_box(T *__restrict__ buf, int nx, int ny, int nz, int64_t js, int64_t ks, int64_t cs,
                                        int ox, int oy)
{
    const int xpad = 16 * (ny + 4), per_plane = xpad + 4 * nx;
    const int stride = gridDim.x * blockDim.x;
    for (int plane = blockIdx.y; plane < 4 * nz; plane += gridDim.y) {
        T *p = buf + (int64_t)(plane / nz) * cs + (int64_t)(plane % nz) * ks + ox + (int64_t)oy * js;
        for (int r0 = blockIdx.x * blockDim.x + threadIdx.x; r0 < per_plane; r0 += kPadUnroll * stride) {
            int64_t dst[kPadUnroll], src[kPadUnroll];
            bool on[kPadUnroll];
#pragma unroll
            for (int u = 0; u < kPadUnroll; ++u) {
                const int r = r0 + u * stride;
                int x, y;
                if (r < xpad) {  // x padding: 16 columns of every padded row
                    const int k = r & 15;
                    x = k < 8 ? k - 8 : nx + (k - 8);
                    y = (r >> 4) - 2;
                } else {  // y padding: 4 rows of the valid columns
                    const int rr = r - xpad, k = rr / nx;
                    x = rr - k * nx;
                    y = k < 2 ? k - 2 : ny + (k - 2);
                }
                const int xs = x < 0 ? x + nx : (x >= nx ? x - nx : x), ys = y < 0 ? y + ny : (y >= ny ? y - ny : y);
                on[u] = r < per_plane;
                dst[u] = x + (int64_t)y * js;
                src[u] = on[u] ? xs + (int64_t)ys * js : 0;
            }
            T v[kPadUnroll];
#pragma unroll
            for (int u = 0; u < kPadUnroll; ++u) v[u] = p[src[u]];
#pragma unroll
            for (int u = 0; u < kPadUnroll; ++u)
                if (on[u]) p[dst[u]] = v[u];
        }
    }
}

template <typename T>
__global__ void level_pad_kernel(T *__restrict__ buf, int nx, int ny, int nz, int64_t js, int64_t ks, int64_t cs,
                                 int ox, int oy)
{
    pad_box(buf, nx, ny, nz, js, ks, cs, ox, oy);
}

// The same for every box of an ensemble buffer, one box per blockIdx.z.
template <typename T>
__global__ void ens_pad_kernel(T *__restrict__ buf, const EnsBoxDesc *__restrict__ boxes, int64_t cs, int ox)
{
    const EnsBoxDesc &d = boxes[blockIdx.z];
    pad_box(buf + d.base, d.nx, d.ny, d.nz, d.js, d.ks, cs, ox, d.oy);
}

}  // namespace axs
