// Refined patches over a periodic coarse level (the scale path's fine level).
//
// A patch refines one block^3 block of coarse cells by 2 in every direction:
// n = 2*block fine cells per side, spacing dx/2, time step dt/2 (two fine steps
// per coarse step). Patches are cubes of fine cells in a fixed-block layout,
// so the patch that owns any fine cell is found by integer division.
//
// Patch layout: valid fine cell (0,0,0) sits at padded position (8, 4, 4);
// every patch holds a ghost ring of 6 columns in x and 4 rows / planes in y
// and z (plus 2 columns of slack on either side for the TMA boxes), rows are
// padded to whole 32-byte sectors (n + 16 columns: every TMA box and the work
// arena's sweep A domain fit, and strides stay 16-byte multiples), boxes start
// on 128-byte lines, and the patches are stacked along each component plane as
// an ensemble's boxes are.
//
// One fine RK4 step of every patch is the two fused sweeps with explicit
// ghost rings instead of periodic wrap: sweep A runs over the valid cells
// plus a ring of 4 (x, keeping the TMA boxes 16-byte aligned) / 2 (y, z)
// cells, reading psi, Pi on the 6 / 4-wide ring, so that sweep B over the
// valid cells finds d3, d4 on its 2-wide stencil ring. The ring therefore has
// to hold psi, Pi at the step's start time; it is filled first from the
// neighbouring patches (same fine level, same time) and, where no patch owns
// a ring cell, by interpolating the coarse level: quartic Lagrange
// interpolation of coarse cell-centre values in each direction (the 5 coarse
// cells around the fine cell's parent; fine centres sit at -1/4 and +1/4 of a
// coarse cell), and in time between the coarse states at the start and end of
// the coarse step -- cubic Hermite for psi (Pi = dpsi/dtau is its derivative)
// and linear for Pi.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "rk4_ops.cuh"

namespace axs {

int level_geom(int32_t dtype, int nx, int ny, int nz, LevelGeom &g);
int level_fill_ghosts(void *data, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g, int ncomp,
                      cudaStream_t st);
int diag_ghost_boxes(const void *data, int32_t dtype, int nx, int ny, int nz, int ox, int oy, int oz, int64_t js,
                     int64_t ks, int64_t cs, int nboxes, int64_t box_stride, const axs_diag_params *p,
                     axs_diag_result *out, int64_t *list, int64_t capacity, void *scratch, int64_t scratch_bytes,
                     cudaStream_t st);
int64_t diag_scratch_bytes_for(int64_t ncell);
constexpr int kPatchOX = 8, kPatchRY = 4, kPatchRZ = 4;  // padded position of valid (0, 0, 0)
// In the work arena (d3, d4, E, Q) valid x = 0 sits at padded column 12, so
// sweep A's domain x in [-4, n + 4) covers whole 32-byte sectors of every row
// (padded 8 .. n + 16) and no output row leaves a partly written sector.
constexpr int kWorkOX = 12;
constexpr int kRingX = 6, kRingYZ = 4;                    // ghost ring widths the step reads
constexpr int64_t kPatchHeader = 128;

struct PatchGeom {
    int n;           // fine cells per side
    int64_t js, ks;  // row and plane strides
    int64_t box;     // elements of one patch in one component plane (128-byte multiple)
    int64_t plane;   // elements of one component plane (all patches)
};

// capacity: patch slots the component planes are laid out for (0: npatches)
static int patch_geom(int32_t dtype, int n, int npatches, PatchGeom &g, int capacity = 0)
{
    AXS_REQUIRE(dtype == AXS_F32 || dtype == AXS_F64, AXS_ERR_INVALID_ARGUMENT, "bad dtype %d", dtype);
    AXS_REQUIRE(n >= 8 && n % 8 == 0 && n <= 256, AXS_ERR_UNSUPPORTED, "patch side %d must be a multiple of 8 in [8, 256]",
                n);
    // the two-sweep step's work items carry 2 * npatches box numbers in 16 bits
    // (checked where it is used); the fused step takes any count
    AXS_REQUIRE(npatches > 0 && npatches <= (1 << 22), AXS_ERR_INVALID_ARGUMENT, "patch count %d out of range",
                npatches);
    const int64_t line = 128 / (int64_t)dtype_size(dtype), sector = 32 / (int64_t)dtype_size(dtype);
    g.n = n;
    g.js = (kPatchOX + n + kRingX + 2 + sector - 1) / sector * sector;  // n + 16 (n is a multiple of 8)
    g.ks = g.js * (n + 2 * kPatchRY);
    g.box = (g.ks * (n + 2 * kPatchRZ) + line - 1) / line * line;
    AXS_REQUIRE(capacity == 0 || (capacity >= npatches && capacity <= (1 << 22)), AXS_ERR_INVALID_ARGUMENT,
                "patch capacity %d below the patch count %d", capacity, npatches);
    g.plane = g.box * (capacity > npatches ? capacity : npatches);
    return AXS_OK;
}

static int64_t patch_items_bound(const PatchGeom &g, int npatches)
{
    // sweep A domain (n+8) x (n+4) x (n+4) and sweep B n^3, tiles >= 16 x 8, chunks >= 1 plane
    // (sweep A tiles are 40 x 12: at most as many as 16 x 8 tiles)
    const int64_t a = (int64_t)((g.n + 8 + 15) / 16) * ((g.n + 4 + 7) / 8) * (g.n + 4);
    const int64_t b = (int64_t)((g.n + 15) / 16) * ((g.n + 7) / 8) * g.n;
    return (a + b) * npatches;
}

static int64_t patch_table_bytes(const PatchGeom &g, int npatches)
{
    return kPatchHeader + (int64_t)npatches * 2 * sizeof(CUtensorMap) + (int64_t)npatches * 2 * sizeof(EnsBoxDesc) +
           4 * patch_items_bound(g, npatches);
}

// The fused step (one launch per fine step, stage values in shared memory)
// covers this patch size and count; otherwise the two sweeps through the
// 8-component work arena step the patches.
static bool patches_fused(int32_t dtype, int n, int npatches);

// bytes of the work arena: none when the fused step covers the patches
static int64_t patch_work_bytes(const PatchGeom &g, int32_t dtype, int n, int npatches)
{
    return patches_fused(dtype, n, npatches) ? 0 : 8 * g.plane * (int64_t)dtype_size(dtype);
}

static int validate_patches(const axs_patches *p, PatchGeom &g)
{
    AXS_REQUIRE(p != nullptr, AXS_ERR_INVALID_ARGUMENT, "null patches");
    int rc = patch_geom(p->dtype, p->n, p->npatches, g, p->capacity);
    if (rc) return rc;
    AXS_REQUIRE(p->dx > 0.0, AXS_ERR_INVALID_ARGUMENT, "dx must be positive");
    const int64_t need_work = patch_work_bytes(g, p->dtype, p->n, p->npatches);
    AXS_REQUIRE(p->state && p->table && (p->work || need_work == 0), AXS_ERR_INVALID_ARGUMENT, "null patch buffer");
    AXS_REQUIRE(((uintptr_t)p->state % 128) == 0 && ((uintptr_t)p->work % 128) == 0 && ((uintptr_t)p->table % 128) == 0,
                AXS_ERR_ALIGNMENT, "patch buffers must be 128-byte aligned");
    const int64_t es = (int64_t)dtype_size(p->dtype);
    AXS_REQUIRE(p->state_bytes >= 4 * g.plane * es && p->work_bytes >= need_work &&
                    p->table_bytes >= patch_table_bytes(g, p->npatches),
                AXS_ERR_WORKSPACE, "patch buffer too small");
    return AXS_OK;
}

// ---------------------------------------------------------------- the two sweeps
template <typename T> struct PatchTilings {
    // sweep A: domain x in [-4, n+4) (tiles start on 16-byte boundaries), y, z in [-2, n+2):
    // 40 x 12 tiles cover the 40 x 36 domain of a 32^3 patch exactly
    using LA = SweepLauncher<T, 2, 40, 12, 8, 2, ForwardA, BoxTable, true>;
    // sweep B: the valid cells
    using LB = SweepLauncher<T, 2, 32, 16, 8, 2, ForwardB, BoxTable, true>;
    static constexpr int TXA = 40, TYA = 12, TXB = 32, TYB = 16;
};

// ---------------------------------------------------------------- the fused step
// One RK4 step of a patch without the stage buffers: each CTA owns a TX x TY
// tile of the valid cells and marches in z. Per plane it runs sweep A on the
// tile plus a 2-cell halo (the A region) from a TMA ring of (psi, Pi) planes
// and keeps d3, d4 (A region, 5 planes) and E, Q (tile, 3 planes) in shared
// memory; sweep B follows two planes behind and writes psi, Pi of the step's
// end over the old values. The tiles of one patch form a thread-block cluster
// that advances in lockstep: after every plane of sweep A a cluster barrier
// makes sure no tile still reads (psi, Pi) of the plane sweep B is about to
// overwrite (the A regions of neighbouring tiles overlap). The per-site
// arithmetic is the two sweeps' own (star_laplacian, stage_a, stage_b), so the
// result equals theirs bit for bit, at about a third of the DRAM traffic.
template <typename T> struct Fused {
    // FP32: two sites per thread on 32 x 16 tiles (174 KB of shared memory, one
    // block per SM); 32 x 8 tiles with one site per thread fit two blocks per SM
    // but ran 20 % slower on GB300. FP64: one site per thread on 32 x 8 tiles.
    // NSW / NGP: d3, d4 and E, Q slots, one more than sweep B reads, so sweep A of
    // the next plane never overwrites what a slower thread's sweep B still reads
    static constexpr int V = sizeof(T) == 4 ? 2 : 1;
    static constexpr int TX = 32, TY = sizeof(T) == 4 ? 16 : 8, NS = sizeof(T) == 4 ? 6 : 5;
    static constexpr int NSW = 6, NGP = 4;
    static constexpr int BX = TX + 8, BY = TY + 8;  // TMA box: the A region plus its stencil halo
    static constexpr int AX = TX + 4, AY = TY + 4;  // A region
    static constexpr int RING = 4 * BX * BY, SWIN = 4 * AX * AY, GPW = 4 * TX * TY;
    static constexpr int NA = AX * AY / V;          // sweep A units (V sites each)
    static_assert(AX / V > 32 / V, "the A region is wider than one bank row");
    static constexpr size_t SMEM = sizeof(T) * ((size_t)NS * RING + NSW * (size_t)SWIN + NGP * (size_t)GPW);
    // 512 threads: sweep A's units run on threads 0 .., sweep B's (one per thread) on the
    // last NB threads, so a plane's critical path is at most one A unit plus one B
    // unit (256 threads: two A units plus one B). Running A and B side by side on
    // separate threads, with B one plane further behind, saturated the shared-memory
    // pipe and ran 10 % slower.
    static constexpr int NB = TX * TY / V;  // sweep B units, one per thread of the last NB threads
    static constexpr int THREADS = 512;
    static_assert(NB <= THREADS, "one sweep B unit per thread");
    static_assert((BX * sizeof(T)) % 16 == 0 && (RING * sizeof(T)) % 128 == 0, "TMA box rows and slots");
    static_assert(SMEM <= 227 * 1024, "shared memory");
};

// tiles of a patch side n (the cluster), or 0 when the fused step does not apply
template <typename T> static void fused_tiles(int n, int &cx, int &cy)
{
    cx = cy = 0;
    if (n % Fused<T>::TX != 0 || n % Fused<T>::TY != 0) return;
    const int x = n / Fused<T>::TX, y = n / Fused<T>::TY;
    if (x * y > 8) return;  // portable cluster size
    cx = x;
    cy = y;
}

static bool patches_fused(int32_t dtype, int n, int npatches)
{
    int cx = 0, cy = 0;
    if (dtype == AXS_F64)
        fused_tiles<double>(n, cx, cy);
    else
        fused_tiles<float>(n, cx, cy);
    return cx > 0;
}

// Execution barrier of the patch's tiles, split so that sweep B's shared-memory
// work runs between arrive and wait. No data passes between the tiles through
// memory: every (psi, Pi) plane a tile reads has landed in its shared memory
// (its TMA transaction completed) before the tile arrives, so the arrive needs
// no release fence.
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.aligned;" ::: "memory"); }

struct FusedArgs {
    int n;
    int q0;  // patch of grid z slice 0 (launches of at most 65 535 patches each)
    int64_t js, ks, box, plane;
    const CUtensorMap *maps;  // per patch q: map 2 q + 1 boxes BX x BY of the state
};

template <typename T>
__global__ void __launch_bounds__(Fused<T>::THREADS, 1) patch_fused_kernel(T *__restrict__ st, const SweepArgs<T> a,
                                                              const FusedArgs f)
{
    using F = Fused<T>;
    constexpr int V = F::V;
    extern __shared__ __align__(128) unsigned char fused_smem[];
    T *ring = reinterpret_cast<T *>(fused_smem);
    T *swin = ring + (size_t)F::NS * F::RING;
    T *gpw = swin + (size_t)F::NSW * F::SWIN;
    __shared__ uint64_t full[F::NS];
    const int tid = threadIdx.x;
    const int q = f.q0 + (int)blockIdx.z, n = f.n;
    const int x0 = blockIdx.x * F::TX, y0 = blockIdx.y * F::TY;  // tile origin (valid cells)
    const CUtensorMap *map = f.maps + 2 * q + 1;
    if (tid == 0) {
        for (int s = 0; s < F::NS; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
        fence_tensormap_acquire(map);
    }
    __syncthreads();
    // planes z = -4 .. n + 3 (padded plane k = z + 4) pass through the ring, plane k in slot k mod NS;
    // the box starts 4 columns / rows before the tile (padded column x0 + 4: 16-byte aligned)
    const int K = n + 2 * kPatchRZ;
    auto issue = [&](int k) {
        const int slot = k % F::NS;
        mbar_arrive_expect_tx(&full[slot], (uint32_t)(F::RING * sizeof(T)));
        tma_load_4d(ring + (size_t)slot * F::RING, map, kPatchOX - 4 + x0, kPatchRY - 4 + y0, k, 0, &full[slot]);
    };
    if (tid == 0)
        for (int k = 0; k < F::NS && k < K; ++k) issue(k);
    int waited = 0;
    bool ok = true;
    const int bt = tid - (F::THREADS - F::NB);  // sweep B unit of this thread (< 0: none)
    const bool has_b = bt >= 0;
    const int bxl = has_b ? V * (bt % (F::TX / V)) : 0, byl = has_b ? bt / (F::TX / V) : 0;  // tile-local sites
    T *const dst0 = st + (int64_t)q * f.box + (kPatchOX + x0 + bxl) + (int64_t)(kPatchRY + y0 + byl) * f.js;
    // iteration i: sweep A at plane za = i - 2 (reads planes k = i .. i + 4), sweep B at zb = za - 2
    for (int i = 0; i < n + 4; ++i) {
        while (waited <= i + 4) {
            if (!mbar_wait_bounded(&full[waited % F::NS], (uint32_t)((waited / F::NS) & 1), a.wait_polls)) {
                if (ok) atomicOr(a.status, kDevTimeout);
                ok = false;
            }
            ++waited;
        }
        if (ok) {
            const T *pl[5];
#pragma unroll
            for (int d = 0; d < 5; ++d) pl[d] = ring + (size_t)((i + d) % F::NS) * F::RING;
            T *sz = swin + (size_t)(i % F::NSW) * F::SWIN;  // d3, d4 of plane za
            T *gz = gpw + (size_t)(i % F::NGP) * F::GPW;    // E, Q of plane za
            for (int u = tid; u < F::NA; u += F::THREADS) {
                // units of the A region's first 32 / V columns row by row (a warp covers
                // whole 128-byte bank rows, so its shared-memory accesses are conflict-free),
                // then the remaining columns
                constexpr int PR = F::AX / V, MAIN = 32 / V, EDGE = PR - MAIN;
                const int row = u < MAIN * F::AY ? u / MAIN : (u - MAIN * F::AY) / EDGE;
                const int col = u < MAIN * F::AY ? u % MAIN : MAIN + (u - MAIN * F::AY) % EDGE;
                const int lx = 2 + V * col, ly = 2 + row;  // box-local first site
                T lap[4][V], ctr[4][V];
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int co = c * F::BX * F::BY;
                    star_laplacian<T, V>(a, pl[0] + co, pl[1] + co, pl[2] + co, pl[3] + co, pl[4] + co,
                                         ly * F::BX + lx, F::BX, lap[c], ctr[c]);
                }
                T o[8][V];
                stage_a<T, V>(a, lap, ctr, o);
                const int so = (ly - 2) * F::AX + (lx - 2);
#pragma unroll
                for (int c = 0; c < 4; ++c) stv<T, V>(sz + c * F::AX * F::AY + so, o[c]);
                const int tx = lx - 4, ty = ly - 4;  // tile-local; V sites lie all inside or all outside
                if (tx >= 0 && tx < F::TX && ty >= 0 && ty < F::TY) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) stv<T, V>(gz + c * F::TX * F::TY + ty * F::TX + tx, o[4 + c]);
                }
            }
        }
        // sweep B's psi_n, Pi_n at plane zb = za - 2: ring plane k = i, whose slot is
        // refilled after the barrier below
        const int zb = i - 4;
        T pq[8][V];
        if (ok && zb >= 0 && has_b) {
            const T *r0 = ring + (size_t)(i % F::NS) * F::RING + (byl + 4) * F::BX + (bxl + 4);
#pragma unroll
            for (int c = 0; c < 4; ++c) ldv<T, V>(r0 + c * F::BX * F::BY, pq[4 + c]);
        }
        __syncthreads();  // d3, d4, E, Q of plane za are in place; ring plane k = i is read no more
        if (tid == 0 && i + F::NS < K) {
            fence_proxy_async_smem();
            issue(i + F::NS);
        }
        // this tile is done with sweep A at za: (psi, Pi) of plane za - 2 is read no more here
        cluster_arrive();
        T o[4][V];
        if (ok && zb >= 0 && has_b) {
            const T *sp[5];
#pragma unroll
            for (int d = 0; d < 5; ++d) sp[d] = swin + (size_t)((zb + d) % F::NSW) * F::SWIN;  // planes zb-2 .. zb+2
            const T *g = gpw + (size_t)((zb + 2) % F::NGP) * F::GPW;                           // plane zb
            T lap[4][V], ctr[4][V];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int co = c * F::AX * F::AY;
                star_laplacian<T, V>(a, sp[0] + co, sp[1] + co, sp[2] + co, sp[3] + co, sp[4] + co,
                                     (byl + 2) * F::AX + (bxl + 2), F::AX, lap[c], ctr[c]);
                ldv<T, V>(g + c * F::TX * F::TY + byl * F::TX + bxl, pq[c]);
            }
            stage_b<T, V>(a, lap, ctr, pq, o);
        }
        // every tile of the patch is done with sweep A at za: plane zb = za - 2 may be overwritten
        cluster_wait();
        if (ok && zb >= 0 && has_b) {
            T *dst = dst0 + (int64_t)(kPatchRZ + zb) * f.ks;
#pragma unroll
            for (int c = 0; c < 4; ++c) stv<T, V>(dst + c * f.plane, o[c]);
        }
    }
    // a wait expired: no bulk copy may still be landing in shared memory when the block exits
    if (!ok && tid == 0) {
        const int issued = K < n + 4 + F::NS ? K : n + 4 + F::NS;
        for (int k = waited; k < issued; ++k) mbar_wait_bounded(&full[k % F::NS], (uint32_t)((k / F::NS) & 1), 1u << 20);
    }
}

struct PatchTableOut {
    int64_t items_a, items_b;
    int grid_a, grid_b;
};

template <typename T> static int build_patch_table(const axs_patches *p, const PatchGeom &g, cudaStream_t st,
                                                   PatchTableOut &out)
{
    using PT = PatchTilings<T>;
    int ba = 0, bb = 0;
    int rc = PT::LA::blocks_per_sm(ba);
    if (rc) return rc;
    if ((rc = PT::LB::blocks_per_sm(bb))) return rc;
    const int sms = device_sm_count();
    AXS_REQUIRE(sms > 0, AXS_ERR_CUDA, "no CUDA device");
    const int np = p->npatches, n = g.n;
    std::vector<EnsBoxDesc> desc(2 * (size_t)np);
    std::vector<uint32_t> items_a, items_b;
    auto fill = [&](EnsBoxDesc &d, int map_box, int lo_x, int lo_yz, int ext_x, int ext_yz, int tx, int ty,
                    int zchunk) {
        d.nx = ext_x;
        d.ny = ext_yz;
        d.nz = ext_yz;
        d.tiles_x = (ext_x + tx - 1) / tx;
        d.ntiles = d.tiles_x * ((ext_yz + ty - 1) / ty);
        d.zchunk = zchunk;
        d.js = g.js;
        d.ks = g.ks;
        d.base = (int64_t)map_box * g.box;
        d.xlo = lo_x;
        d.ylo = d.zlo = lo_yz;
        d.oy = kPatchRY;
        d.oz = kPatchRZ;
        d.periodic = 0;
        d.map_box = map_box;
        d.pad = 0;
    };
    // chunk length: two chunks per patch side, at least 8 planes (a chunk
    // re-reads 4 halo planes; on GB300 two chunks ran 3 % faster than four,
    // and whole patch heights 30 % slower -- neighbouring tiles then march at
    // different heights and miss each other's halo rows in L2)
    const int zc_a = std::max(8, (n + 4 + 1) / 2), zc_b = std::max(8, (n + 1) / 2);
    for (int q = 0; q < np; ++q) {
        fill(desc[q], q, -4, -2, n + 8, n + 4, PT::TXA, PT::TYA, zc_a);
        fill(desc[np + q], q, 0, 0, n, n, PT::TXB, PT::TYB, zc_b);
    }
    // work items of the two-sweep step (the fused step needs none)
    const bool fused = patches_fused(p->dtype, n, np);
    AXS_REQUIRE(fused || 2 * np < (1 << (32 - kEnsItemBits)), AXS_ERR_UNSUPPORTED,
                "%d patches of side %d: the two-sweep step takes fewer than %d", np, n, (1 << (32 - kEnsItemBits)) / 2);
    for (int q = 0; q < np && !fused; ++q) {
        const EnsBoxDesc &da = desc[q], &db = desc[np + q];
        const int64_t na = (int64_t)da.ntiles * ((da.nz + da.zchunk - 1) / da.zchunk);
        const int64_t nb = (int64_t)db.ntiles * ((db.nz + db.zchunk - 1) / db.zchunk);
        for (int64_t i = 0; i < na; ++i) items_a.push_back(((uint32_t)q << kEnsItemBits) | (uint32_t)i);
        for (int64_t i = 0; i < nb; ++i) items_b.push_back(((uint32_t)(np + q) << kEnsItemBits) | (uint32_t)i);
    }
    const size_t maps_off = kPatchHeader, desc_off = maps_off + 2 * sizeof(CUtensorMap) * np,
                 items_off = desc_off + sizeof(EnsBoxDesc) * 2 * np;
    std::vector<unsigned char> img(items_off + 4 * (items_a.size() + items_b.size()), 0);
    const int64_t es = (int64_t)dtype_size(p->dtype);
    for (int q = 0; q < np; ++q) {
        auto *maps = reinterpret_cast<CUtensorMap *>(img.data() + maps_off) + 2 * q;
        const char *sb = static_cast<const char *>(p->state) + (int64_t)q * g.box * es;
        const char *wb = fused ? nullptr : static_cast<const char *>(p->work) + (int64_t)q * g.box * es;
        // sweep A boxes are TXA+8 x TYA+4, sweep B boxes TXB+8 x TYB+4: one map each
        if ((rc = make_tensor_map_4d(&maps[0], sb, p->dtype, g.js, n + 2 * kPatchRY, n + 2 * kPatchRZ, 4, g.js * es,
                                     g.ks * es, g.plane * es, PT::TXA + 8, PT::TYA + 4, 1, 4)))
            return rc;
        if (fused) {  // the fused step's box over the state
            if ((rc = make_tensor_map_4d(&maps[1], sb, p->dtype, g.js, n + 2 * kPatchRY, n + 2 * kPatchRZ, 4,
                                         g.js * es, g.ks * es, g.plane * es, Fused<T>::BX, Fused<T>::BY, 1, 4)))
                return rc;
        } else if ((rc = make_tensor_map_4d(&maps[1], wb, p->dtype, g.js, n + 2 * kPatchRY, n + 2 * kPatchRZ, 4,
                                            g.js * es, g.ks * es, g.plane * es, PT::TXB + 8, PT::TYB + 4, 1, 4))) {
            return rc;
        }
    }
    std::memcpy(img.data() + desc_off, desc.data(), sizeof(EnsBoxDesc) * desc.size());
    std::memcpy(img.data() + items_off, items_a.data(), 4 * items_a.size());
    std::memcpy(img.data() + items_off + 4 * items_a.size(), items_b.data(), 4 * items_b.size());
    AXS_CUDA_CHECK(cudaMemcpyAsync(p->table, img.data(), img.size(), cudaMemcpyHostToDevice, st));
    AXS_CUDA_CHECK(cudaStreamSynchronize(st));
    out.items_a = (int64_t)items_a.size();
    out.items_b = (int64_t)items_b.size();
    out.grid_a = (int)std::min<int64_t>(out.items_a, (int64_t)ba * sms);
    out.grid_b = (int)std::min<int64_t>(out.items_b, (int64_t)bb * sms);
    return AXS_OK;
}

template <typename T>
static int patch_step_fused(const axs_patches *p, const PatchGeom &g, SweepArgs<T> a, int cx, int cy, cudaStream_t st)
{
    using F = Fused<T>;
    static int attr_done = 0;
    if (!attr_done) {
        AXS_CUDA_CHECK(cudaFuncSetAttribute(patch_fused_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)F::SMEM));
        attr_done = 1;
    }
    FusedArgs f{g.n, 0, g.js, g.ks, g.box, g.plane, a.maps};
    cudaLaunchConfig_t cfg{};
    cfg.blockDim = dim3(F::THREADS, 1, 1);
    cfg.dynamicSmemBytes = F::SMEM;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cx;
    attr[0].val.clusterDim.y = (unsigned)cy;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // patches step independently (each reads and writes only its own box), so a set
    // larger than the grid's z limit goes in several launches
    for (int q0 = 0; q0 < p->npatches; q0 += 65535) {
        f.q0 = q0;
        cfg.gridDim = dim3((unsigned)cx, (unsigned)cy, (unsigned)std::min(65535, p->npatches - q0));
        AXS_CUDA_CHECK(cudaLaunchKernelEx(&cfg, patch_fused_kernel<T>, static_cast<T *>(p->state), a, f));
    }
    return launch_status("patch fused step");
}

template <typename T>
static int patch_step(const axs_patches *p, const PatchGeom &g, const axs_patch_plan &plan, const axs_background &bg,
                      double tau_i, double t, double dt, cudaStream_t st)
{
    using PT = PatchTilings<T>;
    char *table = static_cast<char *>(p->table);
    const int np = p->npatches;
    SweepArgs<T> a{};
    fill_step_constants(a, p->dx, dt);
    a.ox = kPatchOX;
    a.status = reinterpret_cast<unsigned *>(table);
    a.maps = reinterpret_cast<const CUtensorMap *>(table + kPatchHeader);
    int fcx = 0, fcy = 0;
    fused_tiles<T>(g.n, fcx, fcy);
    if (patches_fused(p->dtype, g.n, np)) {
        a.c1 = stage_coef<T>(bg, tau_i + t);
        a.c2 = stage_coef<T>(bg, tau_i + t + 0.5 * dt);
        a.c4 = stage_coef<T>(bg, tau_i + t + dt);
        return patch_step_fused<T>(p, g, a, fcx, fcy, st);
    }
    a.boxes = reinterpret_cast<const EnsBoxDesc *>(table + kPatchHeader + 2 * sizeof(CUtensorMap) * np);
    const uint32_t *items = reinterpret_cast<const uint32_t *>(a.boxes + 2 * np);
    T *state = static_cast<T *>(p->state), *work = static_cast<T *>(p->work);
    CUtensorMap unused;
    std::memset(&unused, 0, sizeof(unused));
    SweepArgs<T> aa = a;
    aa.items = items;
    aa.n_items = plan.items_a;
    aa.map_sel = 0;
    aa.dox_out = kWorkOX - kPatchOX;  // stencil on the state, outputs to the work arena
    aa.c1 = stage_coef<T>(bg, tau_i + t);
    aa.c2 = stage_coef<T>(bg, tau_i + t + 0.5 * dt);
    for (int c = 0; c < 8; ++c) aa.out[c] = work + c * g.plane;
    int rc = PT::LA::launch(unused, aa, plan.grid_a, st);
    if (rc) return rc;
    SweepArgs<T> ab = a;
    ab.items = items + plan.items_a;
    ab.n_items = plan.items_b;
    ab.map_sel = 1;
    ab.ox = kWorkOX;                   // stencil and pointwise inputs in the work arena,
    ab.dox_out = kPatchOX - kWorkOX;   // outputs to the state
    ab.c2 = aa.c2;
    ab.c4 = stage_coef<T>(bg, tau_i + t + dt);
    for (int c = 0; c < 4; ++c) ab.pt[c] = work + (4 + c) * g.plane;  // E, Q
    // psi_n, Pi_n: the state's rows start kWorkOX - kPatchOX columns later than the
    // work arena's, so these pointers carry that shift (the loads add the work-arena
    // offset of the site)
    for (int c = 0; c < 4; ++c) ab.pt[4 + c] = state + c * g.plane - (kWorkOX - kPatchOX);
    for (int c = 0; c < 4; ++c) ab.out[c] = state + c * g.plane;
    return PT::LB::launch(unused, ab, plan.grid_b, st);
}

// ---------------------------------------------------------------- coarse <-> fine
// Quartic Lagrange weights on coarse nodes -2..2 at offset -1/4 (s = 0) and
// +1/4 (s = 1) from the parent's centre, in coarse-cell units.
struct QuarticWeights {
    double w[2][5];
    float wf[2][5];
};

static QuarticWeights quartic_weights()
{
    QuarticWeights q;
    for (int s = 0; s < 2; ++s) {
        const double xi = s == 0 ? -0.25 : 0.25;
        for (int k = 0; k < 5; ++k) {
            double num = 1.0, den = 1.0;
            for (int m = 0; m < 5; ++m) {
                if (m == k) continue;
                num *= xi - (m - 2);
                den *= (double)(k - m);
            }
            q.w[s][k] = num / den;
            q.wf[s][k] = (float)q.w[s][k];
        }
    }
    return q;
}

struct CoarseView {
    const void *old_state, *new_state;  // level layout (new may equal old)
    int nx, ny, nz;
    int64_t js, ks, cs;
    int ox, oy;
};

__device__ __forceinline__ int pwrap(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

struct FillArgs {
    int n, np;              // fine patch side, patch count
    int nbx, nby, nbz;      // block grid of the coarse level
    const int *patch_block; // 3 per patch
    const int *block_patch; // nbx*nby*nbz -> patch or -1
    int64_t js, ks, box, plane;
    double theta, hdt;      // time fraction in the coarse step, coarse dt
    int valid_too;          // 1: also the valid cells (initialisation)
    const int *patch_list;  // the patches to fill (NULL: all), one launch row of tiles each
    // time blend weights (host-computed): psi = h[0] psi0 + h[1] Pi0 + h[2] psi1 + h[3] Pi1,
    // Pi = h[4] Pi0 + h[5] Pi1 (h[1], h[3] include the coarse dt)
    double hd[6];
    float hf[6];
};

static void fill_time_weights(FillArgs &f)
{
    const double s = f.theta, s2 = s * s, s3 = s2 * s;
    f.hd[0] = 2 * s3 - 3 * s2 + 1;
    f.hd[1] = (s3 - 2 * s2 + s) * f.hdt;
    f.hd[2] = -2 * s3 + 3 * s2;
    f.hd[3] = (s3 - s2) * f.hdt;
    f.hd[4] = 1.0 - s;
    f.hd[5] = s;
    for (int i = 0; i < 6; ++i) f.hf[i] = (float)f.hd[i];
}

// The fill works on tiles of kFillT x kFillT fine columns of one patch (one CTA
// per tile) and marches in z, one coarse parent plane -- two fine planes -- at
// a time. Quartic interpolation is separable, so the two fine planes are made
// from the tile's coarse footprint (kFillC x kFillC coarse cells: the parents
// plus 2 on either side) in three passes through shared memory: z (5 coarse
// planes -> the footprint at both fine heights), x (-> fine columns x coarse
// rows), y (-> fine cells). Both children of a parent use the same five
// inputs on every axis, so each pass computes them together. The coarse planes
// pass through a 5-slot window, each loaded once per tile with the time
// interpolation already applied (it is linear, so it commutes with the spatial
// one): per coarse cell, psi(theta) is the cubic Hermite blend of psi and
// hdt * Pi at the two ends of the coarse step, Pi(theta) the linear blend of Pi.
constexpr int kFillT = 16;
constexpr int kFillC = kFillT / 2 + 4;
constexpr int kFillCells = kFillC * kFillC;
constexpr int kFillThreads = 256;
constexpr int kFillWin = 4 * kFillCells;            // one window slot: 4 components
constexpr int kFillXs = 4 * kFillC * kFillT;        // one fine plane of x-interpolated rows
static_assert(2 * kFillCells <= 2 * kFillThreads, "coarse load tasks: two per thread");
static_assert(kFillWin <= 3 * kFillThreads && 2 * kFillXs / 2 <= 3 * kFillThreads, "z / x tasks: three per thread");
static_assert(kFillThreads == 2 * kFillT * kFillT / 2, "one y pair of one fine plane per thread");

// Coarse planes are staged raw by cp.async kFillAhead parents ahead of the
// plane the window takes next, in kFillAhead + 1 staging slots: per load task
// psi_pair and Pi_pair at the start of the coarse step and, when blending, at
// its end.
constexpr int kFillAhead = 2;
constexpr int kFillStage = kFillAhead + 1;

template <typename T> struct FillSmem {
    T win[5][kFillWin];                         // coarse plane p sits in slot p mod 5
    T zs[2][kFillWin];                          // footprint interpolated to the two fine heights
    T xs[2][kFillXs];                           // then to the tile's fine columns
    T stage[kFillStage][4][2 * kFillCells];     // raw plane p in slot p mod kFillStage
};

// tiles start at fine x, y = -8 and cover [-kRingX, n + kRingX) x [-kRingYZ, n + kRingYZ)
__host__ __device__ __forceinline__ int fill_tiles_x(int n) { return (n + 8 + kRingX + kFillT - 1) / kFillT; }
__host__ __device__ __forceinline__ int fill_tiles_y(int n) { return (n + 8 + kRingYZ + kFillT - 1) / kFillT; }

// One element, global -> shared by cp.async, to the 32-bit shared address dst + OFF.
template <int BYTES, uint32_t OFF> __device__ __forceinline__ void cp_async_to(uint32_t dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0+%2], [%1], %3;\n" ::"r"(dst), "l"(src), "n"(OFF), "n"(BYTES)
                 : "memory");
}

template <typename T>
__global__ void __launch_bounds__(kFillThreads, sizeof(T) == 4 ? 4 : 2) patch_fill_kernel(T *__restrict__ st, CoarseView cv, FillArgs f,
                                                                     QuarticWeights q)
{
    extern __shared__ __align__(16) unsigned char fill_smem_raw[];  // FillSmem<T>, sizeof bytes
    FillSmem<T> &sm = *reinterpret_cast<FillSmem<T> *>(fill_smem_raw);
    __shared__ T w[2][5];
    const int n = f.n, half = n / 2, tid = threadIdx.x;
    const int ntx = fill_tiles_x(n), ntiles = ntx * fill_tiles_y(n);
    const int li = blockIdx.x / ntiles, tile = blockIdx.x % ntiles;
    const int pq = f.patch_list != nullptr ? f.patch_list[li] : li;
    if (pq < 0 || pq >= f.np) return;  // a list entry outside the patches (whole block: no barrier skipped)
    // tile origins are even, so a fine cell's child index on each axis is its parity
    const int x0 = -8 + kFillT * (tile % ntx), y0 = -8 + kFillT * (tile / ntx);
    const int bx = f.patch_block[3 * pq], by = f.patch_block[3 * pq + 1], bz = f.patch_block[3 * pq + 2];
    const int cx0 = bx * half + x0 / 2 - 2, cy0 = by * half + y0 / 2 - 2;  // footprint origin (unwrapped)
    if (tid == 0) {
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                if constexpr (sizeof(T) == 4)
                    w[a][k] = q.wf[a][k];
                else
                    w[a][k] = q.w[a][k];
            }
    }

    // ---- this thread's cells: fine column pair (x, ya), (x, ya + 1) in plane sz of each parent.
    // ya is even, so both share the block, the region and the inside tests.
    const int sz = tid >> 7, tx = tid & 15, m = (tid >> 4) & 7;
    const int x = x0 + tx, ya = y0 + 2 * m;
    const bool col_region = x >= -kRingX && x < n + kRingX && ya >= -kRingYZ && ya < n + kRingYZ;
    const bool col_inside = x >= 0 && x < n && ya >= 0 && ya < n;
    const bool tile_inside = x0 >= 0 && x0 + kFillT <= n && y0 >= 0 && y0 + kFillT <= n;
    const int gx = pwrap(bx * n + x, cv.nx * 2), gya = pwrap(by * n + ya, cv.ny * 2);
    // the patches owning the column pair's cells below, inside and above this patch in z
    int own_lo = -1, own_mid = -1, own_hi = -1;
    if (col_region && !f.valid_too) {
        const int ob = (gx / n) + f.nbx * (gya / n), bplane = f.nbx * f.nby;
        own_lo = f.block_patch[ob + bplane * pwrap(bz - 1, f.nbz)];
        own_mid = f.block_patch[ob + bplane * bz];
        own_hi = f.block_patch[ob + bplane * pwrap(bz + 1, f.nbz)];
    }
    T *const dst_col = st + (int64_t)pq * f.box + (x + kPatchOX) + (int64_t)(ya + kPatchRY) * f.js;
    const int64_t src_col = (gx % n + kPatchOX) + (int64_t)(gya % n + kPatchRY) * f.js;

    // ---- coarse load tasks (two per thread at most): (pair, cell) -> psi_pair, Pi_pair
    int64_t ld_off[2];
    int ld_sm[2];
    bool ld_on[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int t = tid + r * kFillThreads;
        ld_on[r] = t < 2 * kFillCells;
        const int pair = t / kFillCells, cell = t % kFillCells;
        const int xx = pwrap(cx0 + cell % kFillC, cv.nx), yy = pwrap(cy0 + cell / kFillC, cv.ny);
        ld_off[r] = (int64_t)(yy + cv.oy) * cv.js + cv.ox + xx + (pair ? cv.cs : 0);
        ld_sm[r] = pair * kFillCells + cell;
    }
    // ---- z pass tasks: component-cell of the footprint, both heights
    int zt[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const int t = tid + r * kFillThreads;
        zt[r] = t < kFillWin ? t : -1;
    }
    // ---- x pass tasks: (height, component, coarse row, fine column pair)
    int xin[3], xout[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const int t = tid + r * kFillThreads;
        const int h = t / (kFillXs / 2), rem = t % (kFillXs / 2);
        const int c = rem / (kFillC * kFillT / 2), rem2 = rem % (kFillC * kFillT / 2);
        const int cyl = rem2 / (kFillT / 2), mm = rem2 % (kFillT / 2);
        const bool on = t < kFillXs;
        xin[r] = on ? h * kFillWin + c * kFillCells + cyl * kFillC + mm : -1;
        xout[r] = h * kFillXs + c * kFillC * kFillT + cyl * kFillT + 2 * mm;
    }

    const T *c0 = static_cast<const T *>(cv.old_state), *c1 = static_cast<const T *>(cv.new_state);
    // time blend in the field precision with host-computed weights (FP64
    // issues at 1/64 of the FP32 rate on GB300, conversions included; the
    // blend is rounded to T when stored anyway)
    const bool blend = f.theta != 0.0;
    const T *hw;
    if constexpr (sizeof(T) == 4)
        hw = f.hf;
    else
        hw = f.hd;
    const T h00 = hw[0], h10 = hw[1], h01 = hw[2], h11 = hw[3], l0 = hw[4], l1 = hw[5];
    // plane p's raw values into the next staging slot (this thread's load tasks;
    // only this thread reads them back, after its own cp.async wait), one group
    // per plane, an empty group past `plast`. Planes are issued and committed in
    // order, so the slots rotate: iss for the next issue, cmt for the next commit.
    constexpr uint32_t kCompBytes = 2 * kFillCells * sizeof(T), kSlotBytes = 4 * kCompBytes;
    const uint32_t stage0 = (uint32_t)__cvta_generic_to_shared(&sm.stage[0][0][0]);
    int iss = 0, cmt = 0;
    auto issue = [&](int p, int plast) {
        if (p <= plast) {
            const int64_t zoff = (int64_t)pwrap(p, cv.nz) * cv.ks;
            const uint32_t sl = stage0 + (uint32_t)iss * kSlotBytes;
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                if (!ld_on[r]) continue;
                const uint32_t d = sl + (uint32_t)ld_sm[r] * (uint32_t)sizeof(T);
                const T *g0 = c0 + (zoff + ld_off[r]);
                cp_async_to<sizeof(T), 0>(d, g0);
                cp_async_to<sizeof(T), kCompBytes>(d, g0 + 2 * cv.cs);
                if (blend) {
                    const T *g1 = c1 + (zoff + ld_off[r]);
                    cp_async_to<sizeof(T), 2 * kCompBytes>(d, g1);
                    cp_async_to<sizeof(T), 3 * kCompBytes>(d, g1 + 2 * cv.cs);
                }
            }
        }
        cp_async_commit();
        iss = iss + 1 == kFillStage ? 0 : iss + 1;
    };
    // plane p from its staging slot into its window slot, time-blended
    auto commit = [&](int p) {
        T *slot = sm.win[pwrap(p, 5)];
        const T(*sg)[2 * kFillCells] = sm.stage[cmt];
        cmt = cmt + 1 == kFillStage ? 0 : cmt + 1;
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            if (!ld_on[r]) continue;
            const int i = ld_sm[r];
            if (!blend) {
                slot[i] = sg[0][i];
                slot[i + 2 * kFillCells] = sg[1][i];
            } else {
                const T p0 = sg[0][i], q0 = sg[1][i], p1 = sg[2][i], q1 = sg[3][i];
                slot[i] = h00 * p0 + h10 * q0 + h01 * p1 + h11 * q1;
                slot[i + 2 * kFillCells] = l0 * q0 + l1 * q1;
            }
        }
    };

    // z segments: the whole height, or only the two z rings above and below a
    // tile that lies inside the valid cells
    const int nseg = (tile_inside && !f.valid_too) ? 2 : 1;
    for (int sg = 0; sg < nseg; ++sg) {
        const int za = nseg == 2 ? (sg == 0 ? -kRingYZ : n) : -kRingYZ;
        const int zb = nseg == 2 ? (sg == 0 ? 0 : n + kRingYZ) : n + kRingYZ;
        const int pa = bz * half + za / 2, pb = bz * half + zb / 2;  // parents of the segment (unwrapped)
        __syncthreads();  // the previous segment is done with the window and the staging slots
        const int plast = pb + 1;  // the last plane the segment's window takes
        iss = cmt = 0;
        for (int p = pa - 2; p < pa + 2; ++p) {
            issue(p, plast);
            cp_async_wait<0>();
            commit(p);
        }
        for (int p = pa + 2; p < pa + 2 + kFillAhead; ++p) issue(p, plast);
        // 0: nothing, 1: copy from the patch owning the cells, 2: interpolate. An
        // initialising fill (valid_too) interpolates every cell: the value depends
        // only on the cell's global position, so a ring cell gets what its owner's
        // valid cell gets in the same launch.
        auto mode_of = [&](int p_, int &z_, int &zone_) {
            z_ = 2 * (p_ - bz * half) + sz;
            zone_ = z_ < 0 ? 0 : (z_ < n ? 1 : 2);
            const int src_patch = zone_ == 0 ? own_lo : (zone_ == 1 ? own_mid : own_hi);
            int md = 0;
            if (col_region && (f.valid_too || !(col_inside && zone_ == 1))) md = src_patch >= 0 ? 1 : 2;
            return md;
        };
        // neighbour copies are loaded one parent ahead (other patches' valid cells,
        // which this launch does not write), so their latency overlaps a parent's work
        T cp[4][2];
        auto load_copy = [&](int z_, int zone_) {
            const int src_patch = zone_ == 0 ? own_lo : (zone_ == 1 ? own_mid : own_hi);
            const T *src = st + (int64_t)src_patch * f.box + src_col + (int64_t)(z_ - (zone_ - 1) * n + kPatchRZ) * f.ks;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                cp[c][0] = src[c * f.plane];
                cp[c][1] = src[c * f.plane + f.js];
            }
        };
        {
            int z_, zone_;
            if (mode_of(pa, z_, zone_) == 1) load_copy(z_, zone_);
        }
        for (int pz = pa; pz < pb; ++pz) {
            cp_async_wait<kFillAhead - 1>();  // plane pz + 2 has landed (this thread's copies)
            commit(pz + 2);
            int z, zone;
            const int mode = mode_of(pz, z, zone);
            const bool any = __syncthreads_or(mode == 2);  // also publishes the committed plane
            // the staging slot of plane pz + 2 + kFillAhead last held plane pz - 1,
            // committed before the barrier above
            issue(pz + 2 + kFillAhead, plast);
            T *dst = dst_col + (int64_t)(z + kPatchRZ) * f.ks;
            if (any) {
                const T *s0 = sm.win[pwrap(pz - 2, 5)], *s1 = sm.win[pwrap(pz - 1, 5)], *s2p = sm.win[pwrap(pz, 5)];
                const T *s3p = sm.win[pwrap(pz + 1, 5)], *s4 = sm.win[pwrap(pz + 2, 5)];
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const int t = zt[r];
                    if (t < 0) continue;
                    const T a0 = s0[t], a1 = s1[t], a2 = s2p[t], a3 = s3p[t], a4 = s4[t];
                    sm.zs[0][t] = w[0][0] * a0 + w[0][1] * a1 + w[0][2] * a2 + w[0][3] * a3 + w[0][4] * a4;
                    sm.zs[1][t] = w[1][0] * a0 + w[1][1] * a1 + w[1][2] * a2 + w[1][3] * a3 + w[1][4] * a4;
                }
                __syncthreads();
                const T *zsf = &sm.zs[0][0];
                T *xsf = &sm.xs[0][0];
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    if (xin[r] < 0) continue;
                    const T *in = zsf + xin[r];
                    const T a0 = in[0], a1 = in[1], a2 = in[2], a3 = in[3], a4 = in[4];
                    xsf[xout[r]] = w[0][0] * a0 + w[0][1] * a1 + w[0][2] * a2 + w[0][3] * a3 + w[0][4] * a4;
                    xsf[xout[r] + 1] = w[1][0] * a0 + w[1][1] * a1 + w[1][2] * a2 + w[1][3] * a3 + w[1][4] * a4;
                }
                __syncthreads();
                if (mode == 2) {
                    const T *xr = xsf + sz * kFillXs + m * kFillT + tx;
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const T *in = xr + c * kFillC * kFillT;
                        const T a0 = in[0], a1 = in[kFillT], a2 = in[2 * kFillT], a3 = in[3 * kFillT],
                                a4 = in[4 * kFillT];
                        dst[c * f.plane] = w[0][0] * a0 + w[0][1] * a1 + w[0][2] * a2 + w[0][3] * a3 + w[0][4] * a4;
                        dst[c * f.plane + f.js] =
                            w[1][0] * a0 + w[1][1] * a1 + w[1][2] * a2 + w[1][3] * a3 + w[1][4] * a4;
                    }
                }
            }
            if (mode == 1) {
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    dst[c * f.plane] = cp[c][0];
                    dst[c * f.plane + f.js] = cp[c][1];
                }
            }
            if (pz + 1 < pb) {
                int z_, zone_;
                if (mode_of(pz + 1, z_, zone_) == 1) load_copy(z_, zone_);
            }
        }
    }
}

// The fill's shared memory is dynamic (36 KB in FP32, 72 KB in FP64): the
// opt-in above 48 KB, once per precision.
template <typename T> static int fill_smem_attr()
{
    static int attr_done = 0;  // setting it twice is harmless
    if (!attr_done) {
        AXS_CUDA_CHECK(cudaFuncSetAttribute(patch_fill_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)sizeof(FillSmem<T>)));
        attr_done = 1;
    }
    return AXS_OK;
}

// Mean of the 8 fine children of every coarse cell a patch covers (amrex::average_down).
template <typename T>
__global__ void patch_average_down_kernel(const T *__restrict__ st, T *__restrict__ coarse, CoarseView cv, FillArgs f)
{
    const int m = f.n / 2;
    const int64_t per = (int64_t)m * m * m, total = per * f.np;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int pq = (int)(idx / per);
        const int64_t r = idx % per;
        const int cx = (int)(r % m), cy = (int)((r / m) % m), cz = (int)(r / ((int64_t)m * m));
        const int bx = f.patch_block[3 * pq], by = f.patch_block[3 * pq + 1], bz = f.patch_block[3 * pq + 2];
        const int gx = bx * m + cx, gy = by * m + cy, gz = bz * m + cz;
        for (int c = 0; c < 4; ++c) {
            double s = 0.0;
            for (int d = 0; d < 8; ++d) {
                const int fx = 2 * cx + (d & 1), fy = 2 * cy + ((d >> 1) & 1), fz = 2 * cz + (d >> 2);
                s += (double)st[c * f.plane + (int64_t)pq * f.box + (fx + kPatchOX) + (int64_t)(fy + kPatchRY) * f.js +
                                (int64_t)(fz + kPatchRZ) * f.ks];
            }
            coarse[c * cv.cs + (gx + cv.ox) + (int64_t)(gy + cv.oy) * cv.js + (int64_t)gz * cv.ks] = (T)(0.125 * s);
        }
    }
}

static int grid_cells(int64_t n)
{
    const int sms = device_sm_count() > 0 ? device_sm_count() : 148;
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 16));
}

static int coarse_view(const axs_level *coarse_old, const axs_level *coarse_new, int32_t dtype, CoarseView &v)
{
    AXS_REQUIRE(coarse_old != nullptr && coarse_old->state != nullptr, AXS_ERR_INVALID_ARGUMENT, "null coarse level");
    AXS_REQUIRE(coarse_old->dtype == dtype, AXS_ERR_INVALID_ARGUMENT, "coarse level and patches differ in dtype");
    LevelGeom g;
    int rc = level_geom(coarse_old->dtype, coarse_old->nx, coarse_old->ny, coarse_old->nz, g);
    if (rc) return rc;
    if (coarse_new) {
        AXS_REQUIRE(coarse_new->state && coarse_new->nx == coarse_old->nx && coarse_new->ny == coarse_old->ny &&
                        coarse_new->nz == coarse_old->nz && coarse_new->dtype == dtype,
                    AXS_ERR_INVALID_ARGUMENT, "coarse old/new levels differ");
    }
    v = CoarseView{coarse_old->state, coarse_new ? coarse_new->state : coarse_old->state, coarse_old->nx,
                   coarse_old->ny, coarse_old->nz, g.js, g.ks, g.cs, g.ox, g.oy};
    return AXS_OK;
}

static int fill_args(const axs_patches *p, const PatchGeom &g, const axs_patch_map *m, const CoarseView &cv,
                     FillArgs &f)
{
    AXS_REQUIRE(m != nullptr && m->patch_block != nullptr && m->block_patch != nullptr, AXS_ERR_INVALID_ARGUMENT,
                "null patch map");
    AXS_REQUIRE(g.n % 2 == 0 && cv.nx * 2 % g.n == 0 && cv.ny * 2 % g.n == 0 && cv.nz * 2 % g.n == 0,
                AXS_ERR_UNSUPPORTED, "the coarse level must tile into blocks of %d cells", g.n / 2);
    f.n = g.n;
    f.np = p->npatches;
    f.nbx = cv.nx * 2 / g.n;
    f.nby = cv.ny * 2 / g.n;
    f.nbz = cv.nz * 2 / g.n;
    f.patch_block = m->patch_block;
    f.block_patch = m->block_patch;
    f.js = g.js;
    f.ks = g.ks;
    f.box = g.box;
    f.plane = g.plane;
    f.theta = 0.0;
    f.hdt = 0.0;
    f.valid_too = 0;
    f.patch_list = nullptr;
    return AXS_OK;
}

// Whole patch boxes (4 components) of dst from src: box q from src box
// src_of_dst[q], or zeros where that is negative (or not a src patch), in
// 16-byte words. One launch row per dst patch (grid y strides over them).
__global__ void patch_copy_boxes_kernel(uint4 *__restrict__ dst, const uint4 *__restrict__ src,
                                        const int *__restrict__ src_of_dst, int np_dst, int np_src, int units,
                                        int64_t dst_plane, int64_t src_plane)
{
    for (int q = blockIdx.y; q < np_dst; q += gridDim.y) {
        const int s = src_of_dst[q];
        if (s == AXS_PATCH_KEEP) continue;  // the box stays as it is
        const bool copy = src != nullptr && s >= 0 && s < np_src;
        for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < 4 * units; u += gridDim.x * blockDim.x) {
            const int c = u / units, r = u - c * units;
            const uint4 v = copy ? src[c * src_plane + (int64_t)s * units + r] : make_uint4(0u, 0u, 0u, 0u);
            dst[c * dst_plane + (int64_t)q * units + r] = v;
        }
    }
}

}  // namespace axs

using namespace axs;

extern "C" {

int axs_patches_layout(int32_t dtype, int32_t n, int32_t npatches, axs_patch_layout *out)
{
    AXS_REQUIRE(out != nullptr, AXS_ERR_INVALID_ARGUMENT, "null output");
    PatchGeom g;
    int rc = patch_geom(dtype, n, npatches, g);
    if (rc) return rc;
    const int64_t es = (int64_t)dtype_size(dtype);
    out->jstride = g.js;
    out->kstride = g.ks;
    out->patch_elems = g.box;
    out->plane_elems = g.plane;
    out->x_offset = kPatchOX;
    out->y_offset = kPatchRY;
    out->z_offset = kPatchRZ;
    out->state_bytes = 4 * g.plane * es;
    out->work_bytes = patch_work_bytes(g, dtype, n, npatches);
    out->table_bytes = patch_table_bytes(g, npatches);
    return AXS_OK;
}

int axs_patches_init(const axs_patches *p, axs_patch_plan *plan, void *stream)
{
    PatchGeom g;
    int rc = validate_patches(p, g);
    if (rc) return rc;
    AXS_REQUIRE(plan != nullptr, AXS_ERR_INVALID_ARGUMENT, "null plan");
    PatchTableOut o{};
    rc = p->dtype == AXS_F32 ? build_patch_table<float>(p, g, (cudaStream_t)stream, o)
                             : build_patch_table<double>(p, g, (cudaStream_t)stream, o);
    if (rc) return rc;
    plan->items_a = o.items_a;
    plan->items_b = o.items_b;
    plan->grid_a = o.grid_a;
    plan->grid_b = o.grid_b;
    return AXS_OK;
}

int axs_patches_rk4_step(const axs_patches *p, const axs_patch_plan *plan, const axs_background *bg, double tau_i,
                         double t, double dt, void *stream)
{
    PatchGeom g;
    int rc = validate_patches(p, g);
    if (rc) return rc;
    AXS_REQUIRE(plan != nullptr && bg != nullptr, AXS_ERR_INVALID_ARGUMENT, "null plan or background");
    AXS_REQUIRE(patches_fused(p->dtype, g.n, p->npatches) || (plan->items_a > 0 && plan->items_b > 0),
                AXS_ERR_INVALID_ARGUMENT, "empty plan (run axs_patches_init)");
    AXS_REQUIRE(std::isfinite(dt) && dt > 0.0, AXS_ERR_INVALID_ARGUMENT, "dt must be positive and finite");
    cudaStream_t st = (cudaStream_t)stream;
    return p->dtype == AXS_F32 ? patch_step<float>(p, g, *plan, *bg, tau_i, t, dt, st)
                               : patch_step<double>(p, g, *plan, *bg, tau_i, t, dt, st);
}

int axs_patches_fill(const axs_patches *p, const axs_patch_map *m, const axs_level *coarse_old,
                     const axs_level *coarse_new, double theta, double coarse_dt, int32_t valid_too, void *stream)
{
    return axs_patches_fill_list(p, m, coarse_old, coarse_new, theta, coarse_dt, valid_too, nullptr,
                                 p != nullptr ? p->npatches : 0, stream);
}

int axs_patches_fill_list(const axs_patches *p, const axs_patch_map *m, const axs_level *coarse_old,
                          const axs_level *coarse_new, double theta, double coarse_dt, int32_t valid_too,
                          const int32_t *patch_list, int32_t count, void *stream)
{
    PatchGeom g;
    int rc = validate_patches(p, g);
    if (rc) return rc;
    CoarseView cv;
    if ((rc = coarse_view(coarse_old, coarse_new, p->dtype, cv))) return rc;
    FillArgs f;
    if ((rc = fill_args(p, g, m, cv, f))) return rc;
    AXS_REQUIRE(theta >= 0.0 && theta <= 1.0, AXS_ERR_INVALID_ARGUMENT, "theta must be in [0, 1]");
    AXS_REQUIRE(theta == 0.0 || coarse_new != nullptr, AXS_ERR_INVALID_ARGUMENT, "theta > 0 needs the new coarse state");
    f.theta = theta;
    f.hdt = coarse_dt;
    f.valid_too = valid_too != 0;
    AXS_REQUIRE(count >= 0 && (patch_list != nullptr || count == p->npatches), AXS_ERR_INVALID_ARGUMENT,
                "a patch count without a list must be npatches");
    f.patch_list = patch_list;
    fill_time_weights(f);
    const QuarticWeights q = quartic_weights();
    if (count == 0) return AXS_OK;
    const int64_t blocks = (int64_t)fill_tiles_x(g.n) * fill_tiles_y(g.n) * count;
    AXS_REQUIRE(blocks < (int64_t)INT32_MAX, AXS_ERR_UNSUPPORTED, "too many patches for one fill launch");
    cudaStream_t st = (cudaStream_t)stream;
    if (p->dtype == AXS_F32) {
        if ((rc = fill_smem_attr<float>())) return rc;
        patch_fill_kernel<float><<<(unsigned)blocks, kFillThreads, sizeof(FillSmem<float>), st>>>(
            static_cast<float *>(p->state), cv, f, q);
    } else {
        if ((rc = fill_smem_attr<double>())) return rc;
        patch_fill_kernel<double><<<(unsigned)blocks, kFillThreads, sizeof(FillSmem<double>), st>>>(
            static_cast<double *>(p->state), cv, f, q);
    }
    return launch_status("patch fill");
}

int axs_patches_copy_boxes(const axs_patches *dst, const axs_patches *src, const int32_t *src_of_dst, void *stream)
{
    PatchGeom g;
    int rc = validate_patches(dst, g);
    if (rc) return rc;
    AXS_REQUIRE(src_of_dst != nullptr, AXS_ERR_INVALID_ARGUMENT, "null patch index");
    int64_t src_plane = 0;
    if (src != nullptr) {
        PatchGeom gs;
        if ((rc = validate_patches(src, gs))) return rc;
        AXS_REQUIRE(src->dtype == dst->dtype && src->n == dst->n, AXS_ERR_INVALID_ARGUMENT,
                    "patches of another size or precision");
        src_plane = gs.plane;
    }
    const int64_t es = (int64_t)dtype_size(dst->dtype);
    AXS_REQUIRE(g.box * es % 16 == 0 && g.plane * es % 16 == 0, AXS_ERR_UNSUPPORTED, "patch boxes of 16-byte words");
    const int units = (int)(g.box * es / 16);
    const unsigned gx = (unsigned)std::min<int64_t>((4 * (int64_t)units + 1023) / 1024, 64);
    const dim3 grid(gx, (unsigned)std::min(dst->npatches, 65535));
    patch_copy_boxes_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
        static_cast<uint4 *>(dst->state), src ? static_cast<const uint4 *>(src->state) : nullptr, src_of_dst,
        dst->npatches, src ? src->npatches : 0, units, g.plane * es / 16, src_plane * es / 16);
    return launch_status("patch box copy");
}

int axs_patches_average_down(const axs_patches *p, const axs_patch_map *m, const axs_level *coarse, void *stream)
{
    PatchGeom g;
    int rc = validate_patches(p, g);
    if (rc) return rc;
    CoarseView cv;
    if ((rc = coarse_view(coarse, nullptr, p->dtype, cv))) return rc;
    FillArgs f;
    if ((rc = fill_args(p, g, m, cv, f))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t total = (int64_t)(g.n / 2) * (g.n / 2) * (g.n / 2) * p->npatches;
    if (p->dtype == AXS_F32)
        patch_average_down_kernel<float><<<grid_cells(total), 256, 0, st>>>(
            static_cast<const float *>(p->state), static_cast<float *>(coarse->state), cv, f);
    else
        patch_average_down_kernel<double><<<grid_cells(total), 256, 0, st>>>(
            static_cast<const double *>(p->state), static_cast<double *>(coarse->state), cv, f);
    if ((rc = launch_status("average down"))) return rc;
    LevelGeom lg;
    level_geom(coarse->dtype, coarse->nx, coarse->ny, coarse->nz, lg);
    return level_fill_ghosts(coarse->state, coarse->dtype, coarse->nx, coarse->ny, coarse->nz, lg, 4, st);
}

int axs_patches_diagnostics_scratch_bytes(int32_t n, int32_t npatches, int64_t *bytes)
{
    AXS_REQUIRE(bytes != nullptr, AXS_ERR_INVALID_ARGUMENT, "null output");
    PatchGeom g;
    int rc = patch_geom(AXS_F32, n, npatches, g);
    if (rc) return rc;
    *bytes = diag_scratch_bytes_for((int64_t)n * n * n * npatches);
    return AXS_OK;
}

int axs_patches_diagnostics(const axs_patches *p, const axs_diag_params *prm, axs_diag_result *out, int64_t *list,
                            int64_t capacity, void *scratch, int64_t scratch_bytes, void *stream)
{
    PatchGeom g;
    int rc = validate_patches(p, g);
    if (rc) return rc;
    AXS_REQUIRE(prm != nullptr && prm->boundary == AXS_BOUNDARY_GHOSTS, AXS_ERR_INVALID_ARGUMENT,
                "patch diagnostics read the rings: boundary must be AXS_BOUNDARY_GHOSTS");
    return diag_ghost_boxes(p->state, p->dtype, g.n, g.n, g.n, kPatchOX, kPatchRY, kPatchRZ, g.js, g.ks, g.plane,
                            p->npatches, g.box, prm, out, list, capacity, scratch, scratch_bytes,
                            (cudaStream_t)stream);
}

int axs_patches_device_status(const axs_patches *p, void *stream)
{
    PatchGeom g;
    int rc = validate_patches(p, g);
    if (rc) return rc;
    unsigned host = 0;
    unsigned *dev = static_cast<unsigned *>(p->table);
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
