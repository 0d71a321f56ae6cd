// Ensembles of independent periodic boxes of uneven sizes, advanced together.
//
// Layout: every box keeps the single-level layout of its size (rk4_level.cu:
// 128-byte aligned rows, x_offset one 128-byte line, 2 padding rows, periodic
// copies written by the producing sweep) and the boxes are stacked along each
// component plane at 128-byte aligned element offsets. Component c of all
// boxes is therefore one contiguous plane, the component stride is the same
// for every box, and a per-site operation written for one level (ForwardA /
// ForwardB, rk4_ops.cuh) runs unchanged on any box once the box's base offset
// is added to its element offset.
//
// Work: the (tile, z-chunk) items of all boxes form one list, ordered by
// descending item cost (longest z-chunk first), box-major and tile-fastest
// within a box. A block looks each item's box up in the device table and
// loads planes through that box's own tensor maps, also in the table. Two
// kinds of tiling run over the list:
//   - the one-pass fused step (level_fused.cuh, FusedBoxes item source): ONE
//     persistent launch per RK4 step plus one launch for the boxes' periodic
//     padding, 8 words per site; steps alternate between the state arena and
//     the work arena's first four planes. Boxes need ny a multiple of the
//     tile height and an even nx (a last, partial tile column is masked);
//   - the two sweeps (sweep.cuh, BoxTable item source): one persistent launch
//     per sweep, 28 words per site, any box shape.
//
// Device table (caller-owned, written once by axs_ensemble_init):
//   [0, 128)                header: status word
//   [128, 128 + 768 nboxes) six CUtensorMaps per box: the two sweeps use maps
//                           2b (state) and 2b + 1 (stage increments d3, d4);
//                           the fused step maps 6b .. 6b + 2 (state) and
//                           6b + 3 .. 6b + 5 (work arena)
//   then                    EnsBoxDesc[nboxes], then uint32 work items
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "level_fused.cuh"

namespace axs {

int level_geom(int32_t dtype, int nx, int ny, int nz, LevelGeom &g);
int level_fill_ghosts(void *data, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g, int ncomp,
                      cudaStream_t st);
int diag_level_box(const void *data, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g,
                   const axs_diag_params *p, axs_diag_result *out, void *scratch, int64_t scratch_bytes,
                   cudaStream_t st);
int64_t diag_scratch_bytes_for(int64_t ncell);

constexpr int64_t kEnsHeader = 128;
constexpr int kEnsMapsPerBox = 6;
constexpr int kEnsMinTX = 16, kEnsMinTY = 4;  // smallest tile of any configuration (item-count bound)
constexpr int kEnsMaxBoxes = 1 << (32 - kEnsItemBits);

struct EnsGeometry {
    std::vector<LevelGeom> g;
    std::vector<int64_t> base;
    int64_t plane = 0;  // elements per component plane
};

static int ens_geometry(int32_t dtype, int nboxes, const int32_t *dims, EnsGeometry &out)
{
    AXS_REQUIRE(dtype == AXS_F32 || dtype == AXS_F64, AXS_ERR_INVALID_ARGUMENT, "bad dtype %d", dtype);
    AXS_REQUIRE(nboxes > 0 && nboxes < kEnsMaxBoxes, AXS_ERR_INVALID_ARGUMENT, "box count %d out of range (1..%d)",
                nboxes, kEnsMaxBoxes - 1);
    AXS_REQUIRE(dims != nullptr, AXS_ERR_INVALID_ARGUMENT, "null box dims");
    const int64_t line = 128 / (int64_t)dtype_size(dtype);
    out.g.resize(nboxes);
    out.base.resize(nboxes);
    int64_t off = 0;
    for (int b = 0; b < nboxes; ++b) {
        const int nx = dims[3 * b], ny = dims[3 * b + 1], nz = dims[3 * b + 2];
        int rc = level_geom(dtype, nx, ny, nz, out.g[b]);
        if (rc) return rc;
        const int64_t tiles_bound = (int64_t)((nx + kEnsMinTX - 1) / kEnsMinTX) * ((ny + kEnsMinTY - 1) / kEnsMinTY) * nz;
        AXS_REQUIRE(tiles_bound < (1 << kEnsItemBits), AXS_ERR_UNSUPPORTED, "box %d (%dx%dx%d) is too large for an "
                    "ensemble work list; advance it as a level", b, nx, ny, nz);
        out.base[b] = off;
        off += (out.g[b].ks * nz + line - 1) / line * line;
    }
    out.plane = off;
    for (auto &g : out.g) g.cs = off;  // every box's component stride is the plane size
    return AXS_OK;
}

static int64_t ens_item_bound(int nboxes, const int32_t *dims)
{
    int64_t n = 0;
    for (int b = 0; b < nboxes; ++b)
        n += (int64_t)((dims[3 * b] + kEnsMinTX - 1) / kEnsMinTX) * ((dims[3 * b + 1] + kEnsMinTY - 1) / kEnsMinTY) *
             dims[3 * b + 2];
    return n;
}

static int64_t ens_table_bytes(int nboxes, const int32_t *dims)
{
    return kEnsHeader + (int64_t)nboxes * kEnsMapsPerBox * sizeof(CUtensorMap) +
           (int64_t)nboxes * sizeof(EnsBoxDesc) + 4 * ens_item_bound(nboxes, dims);
}

static uint64_t ens_key(const axs_ensemble *e, int32_t tile_config, int32_t z_chunk)
{
    // FNV-1a over everything the table depends on
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
        for (int i = 0; i < 8; ++i) {
            h ^= (v >> (8 * i)) & 0xff;
            h *= 1099511628211ull;
        }
    };
    mix((uint64_t)e->dtype);
    mix((uint64_t)e->nboxes);
    for (int i = 0; i < 3 * e->nboxes; ++i) mix((uint64_t)e->dims[i]);
    mix((uint64_t)(uintptr_t)e->state);
    mix((uint64_t)(uintptr_t)e->work);
    mix((uint64_t)(uintptr_t)e->table);
    mix((uint64_t)tile_config);
    mix((uint64_t)z_chunk);
    return h;
}

// Key of the tiling each table currently holds (host side; set by init). A
// plan is usable only while its key is the one last written to its table.
// Per-box diagnostics run on up to kDiagLanes streams side by side (boxes of a
// lane one after another, each lane with its own scratch slice), forked from and
// joined back to the caller's stream with events; under graph capture the lanes
// become parallel branches. Small boxes alone leave most of the GPU idle.
constexpr int kDiagLanes = 8;
struct DiagLanes {
    cudaStream_t s[kDiagLanes];
    cudaEvent_t fork, join[kDiagLanes];
};
static std::mutex g_lanes_mu;
static std::unordered_map<int, DiagLanes> g_lanes;  // per device

static int diag_lanes(DiagLanes *&out)
{
    int dev = 0;
    AXS_CUDA_CHECK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_lanes_mu);
    auto it = g_lanes.find(dev);
    if (it == g_lanes.end()) {
        DiagLanes l;
        for (int i = 0; i < kDiagLanes; ++i) {
            AXS_CUDA_CHECK(cudaStreamCreateWithFlags(&l.s[i], cudaStreamNonBlocking));
            AXS_CUDA_CHECK(cudaEventCreateWithFlags(&l.join[i], cudaEventDisableTiming));
        }
        AXS_CUDA_CHECK(cudaEventCreateWithFlags(&l.fork, cudaEventDisableTiming));
        it = g_lanes.emplace(dev, l).first;
    }
    out = &it->second;
    return AXS_OK;
}

static std::mutex g_table_mu;
static std::unordered_map<const void *, uint64_t> g_table_key;

static void remember_table(const void *table, uint64_t key)
{
    std::lock_guard<std::mutex> lk(g_table_mu);
    g_table_key[table] = key;
}

static bool table_holds(const void *table, uint64_t key)
{
    std::lock_guard<std::mutex> lk(g_table_mu);
    auto it = g_table_key.find(table);
    return it != g_table_key.end() && it->second == key;
}

static int validate_ensemble(const axs_ensemble *e, EnsGeometry &geo)
{
    AXS_REQUIRE(e != nullptr, AXS_ERR_INVALID_ARGUMENT, "null ensemble");
    int rc = ens_geometry(e->dtype, e->nboxes, e->dims, geo);
    if (rc) return rc;
    AXS_REQUIRE(e->dx > 0.0, AXS_ERR_INVALID_ARGUMENT, "dx must be positive");
    AXS_REQUIRE(e->state && e->work && e->table, AXS_ERR_INVALID_ARGUMENT, "null ensemble buffer");
    AXS_REQUIRE(((uintptr_t)e->state % 128) == 0 && ((uintptr_t)e->work % 128) == 0 &&
                    ((uintptr_t)e->table % 128) == 0,
                AXS_ERR_ALIGNMENT, "ensemble buffers must be 128-byte aligned");
    const int64_t es = (int64_t)dtype_size(e->dtype);
    AXS_REQUIRE(e->state_bytes >= 4 * geo.plane * es && e->work_bytes >= 8 * geo.plane * es &&
                    e->table_bytes >= ens_table_bytes(e->nboxes, e->dims),
                AXS_ERR_WORKSPACE, "ensemble buffer too small");
    return AXS_OK;
}

// ---------------------------------------------------------------- tilings
struct EnsRun {
    const axs_ensemble *e;
    const EnsGeometry *geo;
    const axs_ensemble_plan *plan;
    const axs_background *bg;
    double tau_i, t0, dt;
    int nsteps;
    cudaStream_t st;
};

struct EnsTiling {
    const char *name;
    int tx, ty;
    uint32_t box_x, box_y;
    int (*caps)(int &cap_a, int &cap_b);  // resident blocks of each sweep on the device
    int (*run)(const EnsRun &);
    bool fused;  // the one-pass fused step (tensor maps and box constraints of FusedBoxes)
};

// The launch arguments that point into the device table.
template <typename T> static void table_args(SweepArgs<T> &a, const axs_ensemble *e, int64_t n_items)
{
    char *table = static_cast<char *>(e->table);
    a.n_items = n_items;
    a.status = reinterpret_cast<unsigned *>(table);
    a.maps = reinterpret_cast<const CUtensorMap *>(table + kEnsHeader);
    a.boxes = reinterpret_cast<const EnsBoxDesc *>(table + kEnsHeader +
                                                   kEnsMapsPerBox * sizeof(CUtensorMap) * (size_t)e->nboxes);
    a.items = reinterpret_cast<const uint32_t *>(a.boxes + e->nboxes);
}

template <typename T, int V, int TX, int TY, int NS, int MINB, bool HINT = false> struct EnsConfig {
    using LA = SweepLauncher<T, V, TX, TY, NS, MINB, ForwardA, BoxTable, HINT>;
    using LB = SweepLauncher<T, V, TX, TY, NS, MINB, ForwardB, BoxTable, HINT>;

    static int caps(int &cap_a, int &cap_b)
    {
        int ba = 0, bb = 0;
        int rc = LA::blocks_per_sm(ba);
        if (rc) return rc;
        if ((rc = LB::blocks_per_sm(bb))) return rc;
        const int sms = device_sm_count();
        AXS_REQUIRE(sms > 0, AXS_ERR_CUDA, "no CUDA device");
        cap_a = ba * sms;
        cap_b = bb * sms;
        return AXS_OK;
    }

    static int run(const EnsRun &r)
    {
        const axs_ensemble *e = r.e;
        const int64_t P = r.geo->plane;
        SweepArgs<T> a{};
        fill_step_constants(a, e->dx, r.dt);
        a.ox = r.geo->g[0].ox;
        table_args(a, e, r.plan->n_items);
        T *state = static_cast<T *>(e->state), *work = static_cast<T *>(e->work);
        CUtensorMap unused;  // the BoxTable source reads each box's map from the table
        std::memset(&unused, 0, sizeof(unused));
        int rc;
        for (int s = 0; s < r.nsteps; ++s) {
            const double t = r.t0 + s * r.dt;
            SweepArgs<T> aa = a;
            aa.map_sel = 0;
            aa.c1 = stage_coef<T>(*r.bg, r.tau_i + t);
            aa.c2 = stage_coef<T>(*r.bg, r.tau_i + t + 0.5 * r.dt);
            for (int c = 0; c < 8; ++c) aa.out[c] = work + c * P;
            if ((rc = LA::launch(unused, aa, r.plan->grid_a, r.st))) return rc;
            SweepArgs<T> ab = a;
            ab.map_sel = 1;
            ab.c2 = aa.c2;
            ab.c4 = stage_coef<T>(*r.bg, r.tau_i + t + r.dt);
            for (int c = 0; c < 4; ++c) ab.pt[c] = work + (4 + c) * P;  // E, Q
            for (int c = 0; c < 4; ++c) ab.pt[4 + c] = state + c * P;   // psi_n, Pi_n
            for (int c = 0; c < 4; ++c) ab.out[c] = state + c * P;
            if ((rc = LB::launch(unused, ab, r.plan->grid_b, r.st))) return rc;
        }
        return AXS_OK;
    }

    static EnsTiling entry(const char *name)
    {
        return EnsTiling{name, TX, TY, (uint32_t)(TX + 8), (uint32_t)(TY + 4), &caps, &run, false};
    }
};

// The one-pass fused step over every box: per RK4 step one launch of
// level_fused_kernel<S, FusedBoxes> from one state buffer into the other and
// one ens_pad_kernel for the periodic padding of the buffer written. An odd
// step count first copies the state arena (padding included) to the work
// arena, so that the last step writes the state arena.
template <int TX, int TY, int NS, int THREADS> struct EnsFusedConfig {
    using S = LevelFusedShape<TX, TY, NS, THREADS>;

    static int prepare()
    {
        static int smem_set = 0;
        if (!smem_set) {
            AXS_CUDA_CHECK(cudaFuncSetAttribute(level_fused_kernel<S, FusedBoxes>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM));
            smem_set = 1;
        }
        return AXS_OK;
    }

    static int caps(int &cap_a, int &cap_b)
    {
        int rc = prepare();
        if (rc) return rc;
        int bps = 0;
        AXS_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, level_fused_kernel<S, FusedBoxes>,
                                                                     S::THREADS, S::SMEM));
        AXS_REQUIRE(bps > 0, AXS_ERR_UNSUPPORTED, "the fused ensemble step does not fit on this device");
        const int sms = device_sm_count();
        AXS_REQUIRE(sms > 0, AXS_ERR_CUDA, "no CUDA device");
        cap_a = cap_b = bps * sms;
        return AXS_OK;
    }

    static int run(const EnsRun &r)
    {
        const axs_ensemble *e = r.e;
        const int64_t P = r.geo->plane;
        int rc = prepare();
        if (rc) return rc;
        SweepArgs<float> a{};
        fill_step_constants(a, e->dx, r.dt);
        a.ox = r.geo->g[0].ox;
        table_args(a, e, r.plan->n_items);
        float *buf[2] = {static_cast<float *>(e->state), static_cast<float *>(e->work)};
        LevelFusedMaps unused;  // FusedBoxes reads each box's maps from the table
        std::memset(&unused, 0, sizeof(unused));
        int max_nz = 1, max_row = 1;
        for (int b = 0; b < e->nboxes; ++b) {
            const int nx = e->dims[3 * b], ny = e->dims[3 * b + 1], nz = e->dims[3 * b + 2];
            max_nz = std::max(max_nz, nz);
            max_row = std::max(max_row, 16 * (ny + 4) + 4 * nx);
        }
        const dim3 pad_grid((unsigned)std::min(64, (max_row + 256 * kPadUnroll - 1) / (256 * kPadUnroll)),
                            (unsigned)std::min(4 * max_nz, 65535), (unsigned)e->nboxes);
        int first = 0;
        if (r.nsteps & 1) {
            AXS_CUDA_CHECK(cudaMemcpyAsync(buf[1], buf[0], (size_t)(4 * P) * sizeof(float), cudaMemcpyDeviceToDevice,
                                           r.st));
            first = 1;
        }
        for (int s = 0; s < r.nsteps; ++s) {
            const double t = r.t0 + s * r.dt;
            const int src = (s + first) & 1;
            SweepArgs<float> as = a;
            as.map_sel = src;
            as.c1 = stage_coef<float>(*r.bg, r.tau_i + t);
            as.c2 = stage_coef<float>(*r.bg, r.tau_i + t + 0.5 * r.dt);
            as.c4 = stage_coef<float>(*r.bg, r.tau_i + t + r.dt);
            float *dst = buf[src ^ 1];
            for (int c = 0; c < 4; ++c) as.out[c] = dst + c * P;
            level_fused_kernel<S, FusedBoxes><<<r.plan->grid_a, S::THREADS, S::SMEM, r.st>>>(unused, as);
            if ((rc = launch_status("fused ensemble step"))) return rc;
            ens_pad_kernel<float><<<pad_grid, 256, 0, r.st>>>(dst, a.boxes, P, a.ox);
            if ((rc = launch_status("ensemble padding"))) return rc;
        }
        return AXS_OK;
    }

    static EnsTiling entry(const char *name)
    {
        return EnsTiling{name, TX, TY, (uint32_t)S::BX, (uint32_t)S::BY, &caps, &run, true};
    }
};

// Whether every box suits a fused tiling of tile height ty: ny a multiple of
// ty, nx even (the last tile column may be partial, its sites come in pairs).
static bool fused_fits(const int32_t *dims, int nboxes, int ty)
{
    for (int b = 0; b < nboxes; ++b)
        if (dims[3 * b] % 2 != 0 || dims[3 * b + 1] % ty != 0) return false;
    return true;
}

// The default (tile_config 0) is the first entry of its table that suits
// every box: the fused step (0.91 ms per step on a mixed 32^3..128^3
// ensemble on GB300), else the fastest two-sweep tiling there (1.01 ms). The
// 16-wide tiles leave no idle columns on boxes whose width is a multiple of
// 16 but read 96-byte rows.
static const EnsTiling kEnsF32[] = {
    EnsFusedConfig<32, 16, 6, 640>::entry("f32 fused 32x16 ring6 t640"),
    EnsConfig<float, 2, 64, 8, 8, 2>::entry("f32 v2 64x8 ring8"),
    EnsConfig<float, 2, 32, 8, 8, 3>::entry("f32 v2 32x8 ring8"),
    EnsConfig<float, 1, 32, 8, 8, 3>::entry("f32 v1 32x8 ring8"),
    EnsConfig<float, 1, 16, 16, 8, 3>::entry("f32 v1 16x16 ring8"),
    EnsConfig<float, 2, 16, 16, 8, 4>::entry("f32 v2 16x16 ring8"),
    EnsConfig<float, 1, 16, 8, 8, 4>::entry("f32 v1 16x8 ring8"),
    EnsConfig<float, 2, 64, 8, 8, 2, true>::entry("f32 v2 64x8 ring8 l2"),
    EnsConfig<float, 2, 32, 8, 8, 3, true>::entry("f32 v2 32x8 ring8 l2"),
};
static const EnsTiling kEnsF64[] = {
    EnsConfig<double, 1, 32, 8, 6, 2>::entry("f64 v1 32x8 ring6"),
    EnsConfig<double, 1, 16, 16, 6, 2>::entry("f64 v1 16x16 ring6"),
    EnsConfig<double, 1, 16, 8, 6, 3>::entry("f64 v1 16x8 ring6"),
};

static int ens_config_count(int32_t dtype)
{
    if (dtype == AXS_F64) return (int)(sizeof(kEnsF64) / sizeof(kEnsF64[0]));
    if (dtype == AXS_F32) return (int)(sizeof(kEnsF32) / sizeof(kEnsF32[0]));
    return 0;
}

static const EnsTiling *ens_config(int32_t dtype, int32_t id)
{
    const int n = ens_config_count(dtype);
    if (n == 0 || id < 0 || id > n) return nullptr;
    const EnsTiling *tab = dtype == AXS_F64 ? kEnsF64 : kEnsF32;
    return &tab[id == 0 ? 0 : id - 1];
}

// The tiling an ensemble runs for tile_config id: id 0 resolves to the first
// entry that suits its boxes.
static const EnsTiling *ens_config_for(const axs_ensemble *e, int32_t id)
{
    if (id != 0) return ens_config(e->dtype, id);
    const int n = ens_config_count(e->dtype);
    for (int i = 1; i <= n; ++i) {
        const EnsTiling *c = ens_config(e->dtype, i);
        if (!c->fused || fused_fits(e->dims, e->nboxes, c->ty)) return c;
    }
    return nullptr;
}

// Chunk length for every box from one target length: each box splits its nz
// planes into ceil(nz / target) nearly equal chunks.
static int box_zchunk(int nz, int target) { return (nz + (nz + target - 1) / target - 1) / ((nz + target - 1) / target); }

// Automatic target: the candidate whose item list best fills the persistent
// grid (last-wave fill x warm-up overhead of `warm` planes per chunk: 4 for the
// two sweeps; 8 for the fused step, whose chunks restart with 4 planes of
// sweep A alone and 8 extra plane loads).
static int auto_ztarget(const int32_t *dims, int nboxes, int tx, int ty, int cap, double warm)
{
    static const int cand[] = {4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256};
    double best = -1.0;
    int pick = 16;
    for (int zt : cand) {
        double work = 0.0, useful = 0.0, longest = 0.0;
        int64_t items = 0;
        for (int b = 0; b < nboxes; ++b) {
            const int nx = dims[3 * b], ny = dims[3 * b + 1], nz = dims[3 * b + 2];
            const int64_t ntiles = (int64_t)((nx + tx - 1) / tx) * ((ny + ty - 1) / ty);
            const int zc = box_zchunk(nz, std::min(zt, nz));
            const int nch = (nz + zc - 1) / zc;
            items += ntiles * nch;
            work += (double)ntiles * (nz + warm * nch);
            useful += (double)ntiles * nz;
            longest = std::max(longest, (double)zc + warm);
        }
        const int64_t g = std::min<int64_t>(items, cap);
        // greedy bound on the makespan: average load per block plus one longest item
        const double makespan = work / (double)g + longest;
        const double score = useful / ((double)cap * makespan);
        if (score > best + 1e-12) {
            best = score;
            pick = zt;
        }
    }
    return pick;
}

}  // namespace axs

using namespace axs;

extern "C" {

int axs_ensemble_sizes(int32_t dtype, int32_t nboxes, const int32_t *dims, int64_t *state_bytes,
                       int64_t *work_bytes, int64_t *table_bytes)
{
    AXS_REQUIRE(state_bytes && work_bytes && table_bytes, AXS_ERR_INVALID_ARGUMENT, "null output");
    EnsGeometry geo;
    int rc = ens_geometry(dtype, nboxes, dims, geo);
    if (rc) return rc;
    const int64_t es = (int64_t)dtype_size(dtype);
    *state_bytes = 4 * geo.plane * es;
    *work_bytes = 8 * geo.plane * es;
    *table_bytes = ens_table_bytes(nboxes, dims);
    return AXS_OK;
}

int axs_ensemble_box_layout(int32_t dtype, int32_t nboxes, const int32_t *dims, int32_t box, axs_ensemble_box *out)
{
    AXS_REQUIRE(out != nullptr, AXS_ERR_INVALID_ARGUMENT, "null output");
    EnsGeometry geo;
    int rc = ens_geometry(dtype, nboxes, dims, geo);
    if (rc) return rc;
    AXS_REQUIRE(box >= 0 && box < nboxes, AXS_ERR_INVALID_ARGUMENT, "box %d out of range", box);
    out->base = geo.base[box];
    out->jstride = geo.g[box].js;
    out->kstride = geo.g[box].ks;
    out->x_offset = geo.g[box].ox;
    out->y_offset = geo.g[box].oy;
    return AXS_OK;
}

int32_t axs_ensemble_tile_config_count(int32_t dtype) { return ens_config_count(dtype); }

const char *axs_ensemble_tile_config_name(int32_t dtype, int32_t id)
{
    const EnsTiling *c = ens_config(dtype, id);
    return c ? c->name : nullptr;
}

int axs_ensemble_init(const axs_ensemble *e, axs_ensemble_plan *plan, void *stream)
{
    EnsGeometry geo;
    int rc = validate_ensemble(e, geo);
    if (rc) return rc;
    AXS_REQUIRE(plan != nullptr, AXS_ERR_INVALID_ARGUMENT, "null plan");
    const EnsTiling *cfg = ens_config_for(e, plan->tile_config);
    AXS_REQUIRE(cfg != nullptr, AXS_ERR_INVALID_ARGUMENT, "tile_config %d out of range (0..%d)", plan->tile_config,
                ens_config_count(e->dtype));
    AXS_REQUIRE(!cfg->fused || fused_fits(e->dims, e->nboxes, cfg->ty), AXS_ERR_UNSUPPORTED,
                "tiling '%s' needs every box's ny a multiple of %d and nx even", cfg->name, cfg->ty);
    AXS_REQUIRE(plan->z_chunk >= 0, AXS_ERR_INVALID_ARGUMENT, "negative z_chunk");
    int cap_a = 0, cap_b = 0;
    if ((rc = cfg->caps(cap_a, cap_b))) return rc;
    const int nb = e->nboxes;
    const int zt = plan->z_chunk > 0 ? plan->z_chunk
                                     : auto_ztarget(e->dims, nb, cfg->tx, cfg->ty, std::min(cap_a, cap_b),
                                                    cfg->fused ? 8.0 : 4.0);

    // box descriptors
    std::vector<EnsBoxDesc> desc(nb);
    for (int b = 0; b < nb; ++b) {
        const int nx = e->dims[3 * b], ny = e->dims[3 * b + 1], nz = e->dims[3 * b + 2];
        EnsBoxDesc &d = desc[b];
        d.nx = nx;
        d.ny = ny;
        d.nz = nz;
        d.tiles_x = (nx + cfg->tx - 1) / cfg->tx;
        d.ntiles = d.tiles_x * ((ny + cfg->ty - 1) / cfg->ty);
        d.zchunk = box_zchunk(nz, std::min(zt, nz));
        d.js = geo.g[b].js;
        d.ks = geo.g[b].ks;
        d.base = geo.base[b];
        d.xlo = d.ylo = d.zlo = 0;
        d.oy = geo.g[b].oy;
        d.oz = 0;
        d.periodic = 1;
        d.map_box = b;
        d.pad = 0;
    }
    // work items: longest chunks first, then box-major, tile-fastest
    std::vector<int> order(nb);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return desc[x].zchunk > desc[y].zchunk; });
    std::vector<uint32_t> items;
    for (int b : order) {
        const int nch = (desc[b].nz + desc[b].zchunk - 1) / desc[b].zchunk;
        const int64_t n = (int64_t)desc[b].ntiles * nch;
        for (int64_t i = 0; i < n; ++i) items.push_back(((uint32_t)b << kEnsItemBits) | (uint32_t)i);
    }
    AXS_REQUIRE((int64_t)items.size() <= ens_item_bound(nb, e->dims), AXS_ERR_WORKSPACE, "work list overflow");

    // table image: header, tensor maps, descriptors, items
    const size_t maps_off = kEnsHeader, desc_off = maps_off + kEnsMapsPerBox * sizeof(CUtensorMap) * nb,
                 items_off = desc_off + sizeof(EnsBoxDesc) * nb;
    std::vector<unsigned char> img(items_off + 4 * items.size(), 0);
    const int64_t es = (int64_t)dtype_size(e->dtype);
    for (int b = 0; b < nb; ++b) {
        const LevelGeom &g = geo.g[b];
        const int ny = e->dims[3 * b + 1], nz = e->dims[3 * b + 2];
        const char *sbase = static_cast<const char *>(e->state) + geo.base[b] * es;
        const char *wbase = static_cast<const char *>(e->work) + geo.base[b] * es;
        if (cfg->fused) {
            // full box, TY + 4 rows of one component, 2 rows of one component (level_fused.cuh)
            auto *maps = reinterpret_cast<CUtensorMap *>(img.data() + maps_off) + kEnsMapsPerBox * b;
            for (int sel = 0; sel < 2; ++sel) {
                const char *base = sel ? wbase : sbase;
                CUtensorMap *m = maps + 3 * sel;
                const uint64_t d0 = g.js, d1 = ny + 4, sj = g.js * es, sk = g.ks * es, sc = geo.plane * es;
                if ((rc = make_tensor_map_4d(&m[0], base, e->dtype, d0, d1, nz, 4, sj, sk, sc, cfg->box_x, cfg->box_y,
                                             1, 4)) ||
                    (rc = make_tensor_map_4d(&m[1], base, e->dtype, d0, d1, nz, 4, sj, sk, sc, cfg->box_x,
                                             (uint32_t)cfg->ty + 4, 1, 1)) ||
                    (rc = make_tensor_map_4d(&m[2], base, e->dtype, d0, d1, nz, 4, sj, sk, sc, cfg->box_x, 2, 1, 1)))
                    return rc;
            }
            continue;
        }
        auto *maps = reinterpret_cast<CUtensorMap *>(img.data() + maps_off) + 2 * b;
        if ((rc = make_tensor_map_4d(&maps[0], sbase, e->dtype, g.js, ny + 4, nz, 4, g.js * es, g.ks * es,
                                     geo.plane * es, cfg->box_x, cfg->box_y, 1, 4)))
            return rc;
        if ((rc = make_tensor_map_4d(&maps[1], wbase, e->dtype, g.js, ny + 4, nz, 4, g.js * es, g.ks * es,
                                     geo.plane * es, cfg->box_x, cfg->box_y, 1, 4)))
            return rc;
    }
    std::memcpy(img.data() + desc_off, desc.data(), sizeof(EnsBoxDesc) * nb);
    std::memcpy(img.data() + items_off, items.data(), 4 * items.size());
    cudaStream_t st = (cudaStream_t)stream;
    AXS_CUDA_CHECK(cudaMemcpyAsync(e->table, img.data(), img.size(), cudaMemcpyHostToDevice, st));
    AXS_CUDA_CHECK(cudaStreamSynchronize(st));

    plan->n_items = (int64_t)items.size();
    plan->grid_a = (int)std::min<int64_t>(plan->n_items, cap_a);
    plan->grid_b = (int)std::min<int64_t>(plan->n_items, cap_b);
    plan->plane_elems = geo.plane;
    plan->key = ens_key(e, plan->tile_config, plan->z_chunk);
    remember_table(e->table, plan->key);
    return AXS_OK;
}

int axs_ensemble_fill_ghosts(const axs_ensemble *e, void *stream)
{
    EnsGeometry geo;
    int rc = validate_ensemble(e, geo);
    if (rc) return rc;
    const int64_t es = (int64_t)dtype_size(e->dtype);
    for (int b = 0; b < e->nboxes; ++b) {
        void *base = static_cast<char *>(e->state) + geo.base[b] * es;
        if ((rc = level_fill_ghosts(base, e->dtype, e->dims[3 * b], e->dims[3 * b + 1], e->dims[3 * b + 2], geo.g[b],
                                    4, (cudaStream_t)stream)))
            return rc;
    }
    return AXS_OK;
}

int axs_ensemble_rk4_advance(const axs_ensemble *e, const axs_ensemble_plan *plan, const axs_background *bg,
                             double tau_i, double t0, double dt, int32_t nsteps, void *stream)
{
    EnsGeometry geo;
    int rc = validate_ensemble(e, geo);
    if (rc) return rc;
    AXS_REQUIRE(plan != nullptr && bg != nullptr, AXS_ERR_INVALID_ARGUMENT, "null plan or background");
    AXS_REQUIRE(plan->key == ens_key(e, plan->tile_config, plan->z_chunk) && plan->n_items > 0 &&
                    table_holds(e->table, plan->key),
                AXS_ERR_INVALID_ARGUMENT,
                "plan does not match the tiling in this ensemble's table (run axs_ensemble_init)");
    AXS_REQUIRE(nsteps >= 0, AXS_ERR_INVALID_ARGUMENT, "negative step count");
    AXS_REQUIRE(std::isfinite(dt) && dt > 0.0, AXS_ERR_INVALID_ARGUMENT, "dt must be positive and finite");
    if (bg->kind == AXS_BG_EXPANDING) {
        AXS_REQUIRE(bg->a_inv > 1.0, AXS_ERR_INVALID_ARGUMENT, "a_inv must exceed 1");
        AXS_REQUIRE(tau_i + t0 > 0.0, AXS_ERR_INVALID_ARGUMENT, "conformal time must stay positive");
    }
    if (nsteps == 0) return AXS_OK;
    const EnsTiling *cfg = ens_config_for(e, plan->tile_config);
    AXS_REQUIRE(cfg != nullptr, AXS_ERR_INVALID_ARGUMENT, "bad tile_config in plan");
    EnsRun r{e, &geo, plan, bg, tau_i, t0, dt, nsteps, (cudaStream_t)stream};
    return cfg->run(r);
}

int axs_ensemble_diagnostics_scratch_bytes(int32_t nboxes, const int32_t *dims, int64_t *bytes)
{
    AXS_REQUIRE(bytes != nullptr && dims != nullptr && nboxes > 0, AXS_ERR_INVALID_ARGUMENT, "bad arguments");
    int64_t m = 0;
    for (int b = 0; b < nboxes; ++b)
        m = std::max(m, diag_scratch_bytes_for((int64_t)dims[3 * b] * dims[3 * b + 1] * dims[3 * b + 2]));
    *bytes = (m + 255) / 256 * 256 * std::min(nboxes, kDiagLanes);  // one slice per lane
    return AXS_OK;
}

int axs_ensemble_diagnostics(const axs_ensemble *e, const axs_diag_params *p, axs_diag_result *result_dev,
                             void *scratch, int64_t scratch_bytes, void *stream)
{
    EnsGeometry geo;
    int rc = validate_ensemble(e, geo);
    if (rc) return rc;
    AXS_REQUIRE(p != nullptr && result_dev != nullptr, AXS_ERR_INVALID_ARGUMENT, "null params or results");
    int64_t need = 0;
    if ((rc = axs_ensemble_diagnostics_scratch_bytes(e->nboxes, e->dims, &need))) return rc;
    AXS_REQUIRE(scratch != nullptr && scratch_bytes >= need, AXS_ERR_WORKSPACE,
                "ensemble diagnostics scratch too small (%lld < %lld bytes)", (long long)scratch_bytes, (long long)need);
    const int lanes = std::min(e->nboxes, kDiagLanes);
    const int64_t slice = need / lanes;
    DiagLanes *L = nullptr;
    if ((rc = diag_lanes(L))) return rc;
    std::lock_guard<std::mutex> lock(g_lanes_mu);  // the lanes' streams and events are shared: one call at a time
    cudaStream_t st = (cudaStream_t)stream;
    AXS_CUDA_CHECK(cudaEventRecord(L->fork, st));
    // Fork: a lane whose wait could not be recorded is left out of the work and
    // the join (it was never forked). The first CUDA error is kept and returned.
    bool forked[kDiagLanes] = {};
    cudaError_t first = cudaSuccess;
    for (int i = 0; i < lanes; ++i) {
        const cudaError_t e_ = cudaStreamWaitEvent(L->s[i], L->fork, 0);
        forked[i] = e_ == cudaSuccess;
        if (e_ != cudaSuccess && first == cudaSuccess) first = e_;
    }
    const int64_t es = (int64_t)dtype_size(e->dtype);
    for (int b = 0; b < e->nboxes && rc == AXS_OK && first == cudaSuccess; ++b) {
        const int i = b % lanes;
        const void *base = static_cast<const char *>(e->state) + geo.base[b] * es;
        rc = diag_level_box(base, e->dtype, e->dims[3 * b], e->dims[3 * b + 1], e->dims[3 * b + 2], geo.g[b], p,
                            result_dev + b, static_cast<char *>(scratch) + i * slice, slice, L->s[i]);
    }
    // Join every forked lane back, after an error too, so that no lane is left
    // forked from a capturing stream; keep going past a failed join.
    for (int i = 0; i < lanes; ++i) {
        if (!forked[i]) continue;
        cudaError_t e_ = cudaEventRecord(L->join[i], L->s[i]);
        if (e_ == cudaSuccess) e_ = cudaStreamWaitEvent(st, L->join[i], 0);
        if (e_ != cudaSuccess && first == cudaSuccess) first = e_;
    }
    if (first != cudaSuccess) {
        set_error("ensemble diagnostics: fork/join of the lane streams failed: %s", cudaGetErrorString(first));
        return AXS_ERR_CUDA;
    }
    return rc;
}

int axs_ensemble_device_status(const axs_ensemble *e, void *stream)
{
    EnsGeometry geo;
    int rc = validate_ensemble(e, geo);
    if (rc) return rc;
    unsigned host = 0;
    unsigned *dev = static_cast<unsigned *>(e->table);
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
