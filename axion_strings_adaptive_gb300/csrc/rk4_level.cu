// Fused classic-RK4 level advance: two TMA-staged stencil sweeps per step.
//
// Classic RK4 applied to y = (psi, Pi), y' = (Pi, F(t, psi)) with
//   F(t, psi) = lap(psi) + [kappa(t) - lambda(t)/2 (|psi|^2 - R(t)^2)] psi
// (AxionStringsRHS.impl.hpp:44-59) has stage states whose psi parts are
//   psi_n, psi_n + h/2 Pi_n, psi_n + h/2 Pi_n + h^2/4 F1, psi_n + h Pi_n + h^2/2 F2
// so the four stage RHS evaluations pair up:
//   sweep A reads (psi_n, Pi_n) and evaluates F1 = F(t, psi_n),
//                                             F2 = F(t+h/2, psi_n + h/2 Pi_n);
//   sweep B reads (d3, d4)      and evaluates F3 = F(t+h/2, S3), F4 = F(t+h, S4),
// with S3 = psi_n + d3, d3 = h/2 Pi_n + h^2/4 F1, S4 = psi_n + d4,
// d4 = h Pi_n + h^2/2 F2, and
//   psi_{n+1} = psi_n + h Pi_n + h^2/6 (F1 + F2 + F3),
//   Pi_{n+1}  = Pi_n + h/6 F1 + h/3 F2 + h/3 F3 + h/6 F4,
// which is classic RK4 term for term (exact arithmetic). Sweep A stores only
// increments (d3, d4 and the parts E, Q of the two updates known after F1,
// F2; rk4_ops.cuh), so the state is rounded once per step. Per site and step
// the sweeps move 4+8 and 12+4 words: 28 words instead of the 64 of a
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

#include "level_fused.cuh"
#include "rk4_ops.cuh"

namespace axs {

int level_fill_ghosts(void *data, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g, int ncomp,
                      cudaStream_t st);
int level_copy_contiguous(void *lv, void *arr, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g,
                          int to_level, cudaStream_t st);
int level_copy_fab(void *lv, int32_t dtype, const LevelGeom &g, const axs_fab &f, int to_level, cudaStream_t st);

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
    g.ox = line;                                     // x = 0 starts a line; 8 periodic columns sit left of it
    g.oy = 2;
    g.js = ((int64_t)nx + g.ox + 8 + line - 1) / line * line;  // and at least 8 right of x = nx - 1
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
    AXS_REQUIRE((lv->flags & ~AXS_LEVEL_COMPENSATED_FP32) == 0, AXS_ERR_INVALID_ARGUMENT, "unknown level flags 0x%x",
                lv->flags);
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
    void *out_state;  // one whole step into this buffer (level layout), the state unchanged; null: in place
};

// Step constants plus this level's strides and status word.
template <typename T>
static void fill_level_constants(SweepArgs<T> &a, const axs_level *lv, const LevelGeom &g, double dt)
{
    fill_step_constants(a, lv->dx, dt);
    a.js = g.js;
    a.ks = g.ks;
    a.cs = g.cs;
    a.ox = g.ox;
    a.status = level_status_word(lv, g);
}

int make_level_map(CUtensorMap *map, const void *base, int32_t dtype, const LevelGeom &g, int ny, int nz,
                   uint32_t box_x, uint32_t box_y)
{
    const uint64_t es = dtype_size(dtype);
    return make_tensor_map_4d(map, base, dtype, g.js, ny + 4, nz, 4, g.js * es, g.ks * es, g.cs * es, box_x, box_y, 1,
                              4);
}

template <typename T, int V, int TX, int TY, int NS, int MINB, bool HINT = false, bool COMP = false>
struct SweepConfig {
    using LA = SweepLauncher<T, V, TX, TY, NS, MINB, ForwardAT<COMP>, SingleLevel, HINT>;
    using LB = SweepLauncher<T, V, TX, TY, NS, MINB, ForwardBT<COMP>, SingleLevel, HINT>;

    static int run(const SweepRunArgs &r)
    {
        const axs_level *lv = r.lv;
        const LevelGeom &g = *r.g;
        SweepArgs<T> a{};
        int grid = 0, grid_b = 0;
        int rc = LA::plan(a, lv->nx, lv->ny, lv->nz, grid);
        if (rc) return rc;
        SweepArgs<T> tmp = a;
        if ((rc = LB::plan(tmp, lv->nx, lv->ny, lv->nz, grid_b))) return rc;
        fill_level_constants(a, lv, g, r.dt);
        T *state = static_cast<T *>(lv->state), *work = static_cast<T *>(lv->work);
        CUtensorMap map_state, map_work;
        if ((rc = make_level_map(&map_state, state, lv->dtype, g, lv->ny, lv->nz, LA::box_x(), LA::box_y())))
            return rc;
        if ((rc = make_level_map(&map_work, work, lv->dtype, g, lv->ny, lv->nz, LB::box_x(), LB::box_y())))
            return rc;
        for (int s = 0; s < r.nsteps; ++s) {
            const double t = r.t0 + s * r.dt;
            if (r.sweep_mask & 1) {
                SweepArgs<T> aa = a;
                aa.c1 = stage_coef<T>(*r.bg, r.tau_i + t);
                aa.c2 = stage_coef<T>(*r.bg, r.tau_i + t + 0.5 * r.dt);
                for (int c = 0; c < 8; ++c) aa.out[c] = work + c * g.cs;
                if ((rc = LA::launch(map_state, aa, grid, r.st))) return rc;
            }
            if (r.sweep_mask & 2) {
                SweepArgs<T> ab = a;
                ab.n_items = tmp.n_items;
                ab.zchunk = tmp.zchunk;
                ab.c2 = stage_coef<T>(*r.bg, r.tau_i + t + 0.5 * r.dt);
                ab.c4 = stage_coef<T>(*r.bg, r.tau_i + t + r.dt);
                for (int c = 0; c < 4; ++c) ab.pt[c] = work + (4 + c) * g.cs;  // E, Q
                for (int c = 0; c < 4; ++c) ab.pt[4 + c] = state + c * g.cs;   // psi_n, Pi_n
                T *dst = r.out_state != nullptr ? static_cast<T *>(r.out_state) : state;
                for (int c = 0; c < 4; ++c) ab.out[c] = dst + c * g.cs;
                if ((rc = LB::launch(map_work, ab, grid_b, r.st))) return rc;
            }
        }
        return AXS_OK;
    }
};

// The one-pass fused step (level_fused.cuh) over FP32 levels whose extents are
// multiples of its tile; single sweeps and other extents run the two sweeps of
// the fastest two-sweep tiling. Steps alternate between the level's state and
// the first 4 component planes of its work buffer (same layout); each step is
// the fused launch and the padding launch. An odd step count runs its first
// step as the two sweeps, which step the state in place.
template <int TX, int TY, int NS, int THREADS = 512, bool COMP = false> struct FusedConfig {
    using S = LevelFusedShape<TX, TY, NS, THREADS, COMP>;
    using Fallback = SweepConfig<float, 2, 32, 8, 8, 3, true, COMP>;  // the fastest two-sweep tiling at 512^3

    static bool applies(const axs_level *lv)
    {
        return lv->dtype == AXS_F32 && lv->nx % TX == 0 && lv->ny % TY == 0;
    }

    static int maps_for(LevelFusedMaps &m, const float *base, const LevelGeom &g, int ny, int nz)
    {
        const uint64_t es = sizeof(float);
        int rc = make_tensor_map_4d(&m.full, base, AXS_F32, g.js, ny + 4, nz, 4, g.js * es, g.ks * es, g.cs * es,
                                    S::BX, S::BY, 1, 4);
        if (rc) return rc;
        if ((rc = make_tensor_map_4d(&m.mid, base, AXS_F32, g.js, ny + 4, nz, 4, g.js * es, g.ks * es, g.cs * es,
                                     S::BX, TY + 4, 1, 1)))
            return rc;
        return make_tensor_map_4d(&m.rows2, base, AXS_F32, g.js, ny + 4, nz, 4, g.js * es, g.ks * es, g.cs * es,
                                  S::BX, 2, 1, 1);
    }

    static int run(const SweepRunArgs &r)
    {
        const axs_level *lv = r.lv;
        if (r.sweep_mask != 3 || !applies(lv)) return Fallback::run(r);
        // An odd step count takes its first step as the two sweeps (in place; the
        // results are the same bits), so the fused steps after it come in pairs
        // and end in the state buffer. A step into another buffer is one fused
        // launch from the state.
        if ((r.nsteps & 1) && r.out_state == nullptr) {
            SweepRunArgs one = r;
            one.nsteps = 1;
            const int rc1 = Fallback::run(one);
            if (rc1 || r.nsteps == 1) return rc1;
            SweepRunArgs rest = r;
            rest.t0 = r.t0 + r.dt;
            rest.nsteps = r.nsteps - 1;
            return run(rest);
        }
        const LevelGeom &g = *r.g;
        static int smem_set = 0;
        auto kern = level_fused_kernel<S, FusedLevel>;
        if (!smem_set) {
            AXS_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM));
            smem_set = 1;
        }
        const int sms = device_sm_count();
        AXS_REQUIRE(sms > 0, AXS_ERR_CUDA, "no CUDA device");
        SweepArgs<float> a{};
        a.nx = lv->nx;
        a.ny = lv->ny;
        a.nz = lv->nz;
        a.tiles_x = lv->nx / TX;
        a.ntiles = a.tiles_x * (lv->ny / TY);
        // (tile, z-chunk) items taken by blocks in turn: the blocks running at
        // one time march neighbouring tiles through the same planes, so the
        // halo rows they share are L2 hits. (One contiguous tile-major range per
        // block restarted the march less often and balanced the blocks exactly,
        // but was 10 % slower at 512^3: neighbours sat at unrelated planes.)
        int grid = 0;
        plan_chunks(a.ntiles, lv->nz, sms, a.zchunk, a.n_items, grid);
        fill_level_constants(a, lv, g, r.dt);
        const int pad_per_plane = 16 * (lv->ny + 4) + 4 * lv->nx;
        const dim3 pad_grid((unsigned)std::min(64, (pad_per_plane + 256 * kPadUnroll - 1) / (256 * kPadUnroll)),
                            (unsigned)std::min(4 * lv->nz, 65535));
        float *buf[2] = {static_cast<float *>(lv->state),
                         static_cast<float *>(r.out_state != nullptr ? r.out_state : lv->work)};
        LevelFusedMaps maps[2];
        int rc;
        for (int b = 0; b < 2; ++b)
            if ((rc = maps_for(maps[b], buf[b], g, lv->ny, lv->nz))) return rc;
        for (int s = 0; s < r.nsteps; ++s) {
            const double t = r.t0 + s * r.dt;
            SweepArgs<float> as = a;
            as.c1 = stage_coef<float>(*r.bg, r.tau_i + t);
            as.c2 = stage_coef<float>(*r.bg, r.tau_i + t + 0.5 * r.dt);
            as.c4 = stage_coef<float>(*r.bg, r.tau_i + t + r.dt);
            float *dst = buf[(s + 1) & 1];
            for (int c = 0; c < 4; ++c) as.out[c] = dst + c * g.cs;
            kern<<<grid, S::THREADS, S::SMEM, r.st>>>(maps[s & 1], as);
            if ((rc = launch_status("fused level step"))) return rc;
            level_pad_kernel<float><<<pad_grid, 256, 0, r.st>>>(dst, lv->nx, lv->ny, lv->nz, g.js, g.ks, g.cs, g.ox, g.oy);
            if ((rc = launch_status("level padding"))) return rc;
        }
        return AXS_OK;
    }
};

// Tile configurations (vector width, tile, ring depth, expected blocks/SM).
// Entry 0 of each table is the default (tile_config = 0). run_comp: the
// compensated FP32 step (AXS_LEVEL_COMPENSATED_FP32) of the same tiling, where
// one is compiled; other tilings run the default entry's.
struct TileConfigEntry {
    const char *name;
    int (*run)(const SweepRunArgs &);
    int (*run_comp)(const SweepRunArgs &);
};

static const TileConfigEntry kF32Configs[] = {
    // the default: the fastest FP32 step at 512^3 (two sweeps where it does not apply)
    {"f32 fused 32x16 ring6 t640", &FusedConfig<32, 16, 6, 640>::run, &FusedConfig<32, 16, 6, 640, true>::run},
    {"f32 v2 64x8 ring8", &SweepConfig<float, 2, 64, 8, 8, 2>::run, nullptr},
    {"f32 v2 32x16 ring8", &SweepConfig<float, 2, 32, 16, 8, 2>::run, nullptr},
    {"f32 v4 32x16 ring8", &SweepConfig<float, 4, 32, 16, 8, 2>::run, nullptr},
    {"f32 v2 32x8 ring8", &SweepConfig<float, 2, 32, 8, 8, 3>::run, nullptr},
    {"f32 v1 32x8 ring8", &SweepConfig<float, 1, 32, 8, 8, 3>::run, nullptr},
    {"f32 v2 64x8 ring10", &SweepConfig<float, 2, 64, 8, 10, 1>::run, nullptr},
    {"f32 v4 64x16 ring6", &SweepConfig<float, 4, 64, 16, 6, 1>::run, nullptr},
    {"f32 v2 32x16 ring6", &SweepConfig<float, 2, 32, 16, 6, 2>::run, nullptr},
    {"f32 v1 32x16 ring7", &SweepConfig<float, 1, 32, 16, 7, 2>::run, nullptr},
    // L2 policies: stencil planes evict-last, pointwise inputs and outputs evict-first
    {"f32 v2 64x8 ring8 l2", &SweepConfig<float, 2, 64, 8, 8, 2, true>::run, nullptr},
    {"f32 v2 32x16 ring8 l2", &SweepConfig<float, 2, 32, 16, 8, 2, true>::run, nullptr},
    {"f32 v2 32x8 ring8 l2", &SweepConfig<float, 2, 32, 8, 8, 3, true>::run,
     &SweepConfig<float, 2, 32, 8, 8, 3, true, true>::run},
    {"f32 v4 64x16 ring6 l2", &SweepConfig<float, 4, 64, 16, 6, 1, true>::run, nullptr},
    // one-pass fused step (level_fused.cuh)
    {"f32 fused 32x16 ring6", &FusedConfig<32, 16, 6>::run, nullptr},
    {"f32 fused 32x16 ring7", &FusedConfig<32, 16, 7>::run, nullptr},
    {"f32 fused 32x16 ring7 t640", &FusedConfig<32, 16, 7, 640>::run, nullptr},
};
static const TileConfigEntry kF64Configs[] = {
    {"f64 v1 32x8 ring6", &SweepConfig<double, 1, 32, 8, 6, 2>::run, nullptr},
    {"f64 v2 32x8 ring6", &SweepConfig<double, 2, 32, 8, 6, 2>::run, nullptr},
    {"f64 v2 32x16 ring6", &SweepConfig<double, 2, 32, 16, 6, 1>::run, nullptr},
    {"f64 v1 32x4 ring7", &SweepConfig<double, 1, 32, 4, 7, 3>::run, nullptr},
    {"f64 v1 32x8 ring6 l2", &SweepConfig<double, 1, 32, 8, 6, 2, true>::run, nullptr},
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

// The level's runner: its tiling, or the compensated FP32 step when the level
// asks for it (FP64 levels have no compensated form: the flag changes nothing).
using Runner = int (*)(const SweepRunArgs &);
static Runner runner_for(const axs_level *lv, const TileConfigEntry *cfg)
{
    if (lv->dtype == AXS_F32 && (lv->flags & AXS_LEVEL_COMPENSATED_FP32))
        return cfg->run_comp != nullptr ? cfg->run_comp : kF32Configs[0].run_comp;
    return cfg->run;
}

static int run_sweeps(const axs_level *lv, const LevelGeom &g, const axs_background *bg, double tau_i, double t0,
                      double dt, int nsteps, int mask, cudaStream_t st)
{
    const TileConfigEntry *cfg = config_for(lv->dtype, lv->tile_config);
    AXS_REQUIRE(cfg != nullptr, AXS_ERR_INVALID_ARGUMENT, "tile_config %d out of range (0..%d)", lv->tile_config,
                config_count(lv->dtype));
    SweepRunArgs r{lv, &g, bg, tau_i, t0, dt, nsteps, mask, st, nullptr};
    return runner_for(lv, cfg)(r);
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

// Host <-> level copies as one 3D copy each: the host array (4, nz, ny, nx) is
// 4*nz slices of ny rows of nx elements; in the level a slice is kstride
// elements (jstride * (ny + 4)) and the component stride is nz slices, so slice
// c*nz + z lands on component c, plane z.
// Host transfers go through the level's work buffer as a contiguous staging
// array: one plain DMA copy of the whole state each way (the link runs ~20 %
// faster on one contiguous copy than on the row-strided copy straight into
// the padded layout), plus one device pass between the staging array and the
// level layout. The work buffer holds only stage values inside a step, so it
// is free between steps; its status block (after the 8 components) is left alone.
int axs_level_upload(const axs_level *lv, const void *host_state, void *stream)
{
    LevelGeom g;
    int rc = validate_level(lv, g);
    if (rc) return rc;
    AXS_REQUIRE(host_state != nullptr, AXS_ERR_INVALID_ARGUMENT, "null host state");
    const size_t bytes = (size_t)4 * lv->nx * lv->ny * lv->nz * dtype_size(lv->dtype);
    AXS_CUDA_CHECK(cudaMemcpyAsync(lv->work, host_state, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    return level_copy_contiguous(lv->state, lv->work, lv->dtype, lv->nx, lv->ny, lv->nz, g, 1, (cudaStream_t)stream);
}

int axs_level_download(const axs_level *lv, void *host_state, void *stream)
{
    LevelGeom g;
    int rc = validate_level(lv, g);
    if (rc) return rc;
    AXS_REQUIRE(host_state != nullptr, AXS_ERR_INVALID_ARGUMENT, "null host state");
    rc = level_copy_contiguous(lv->state, lv->work, lv->dtype, lv->nx, lv->ny, lv->nz, g, 0, (cudaStream_t)stream);
    if (rc) return rc;
    const size_t bytes = (size_t)4 * lv->nx * lv->ny * lv->nz * dtype_size(lv->dtype);
    AXS_CUDA_CHECK(cudaMemcpyAsync(host_state, lv->work, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    return AXS_OK;
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

int axs_level_rk4_step_to(const axs_level *lv, void *dst_state, const axs_background *bg, double tau_i, double t,
                          double dt, void *stream)
{
    LevelGeom g;
    int rc = validate_level(lv, g);
    if (rc) return rc;
    AXS_REQUIRE(bg != nullptr, AXS_ERR_INVALID_ARGUMENT, "null background");
    AXS_REQUIRE(std::isfinite(dt) && dt > 0.0, AXS_ERR_INVALID_ARGUMENT, "dt must be positive and finite");
    AXS_REQUIRE(dst_state != nullptr, AXS_ERR_INVALID_ARGUMENT, "null destination state");
    AXS_REQUIRE(((uintptr_t)dst_state % 128) == 0, AXS_ERR_ALIGNMENT, "destination state must be 128-byte aligned");
    const size_t bytes = 4 * (size_t)g.cs * dtype_size(lv->dtype);
    const char *d = static_cast<const char *>(dst_state), *s0 = static_cast<const char *>(lv->state),
               *w0 = static_cast<const char *>(lv->work);
    AXS_REQUIRE(d + bytes <= s0 || d >= s0 + bytes, AXS_ERR_INVALID_ARGUMENT, "destination overlaps the state");
    AXS_REQUIRE(d + bytes <= w0 || d >= w0 + 8 * (size_t)g.cs * dtype_size(lv->dtype) + 256, AXS_ERR_INVALID_ARGUMENT,
                "destination overlaps the work buffer");
    if (bg->kind == AXS_BG_EXPANDING) {
        AXS_REQUIRE(bg->a_inv > 1.0, AXS_ERR_INVALID_ARGUMENT, "a_inv must exceed 1");
        AXS_REQUIRE(tau_i + t > 0.0, AXS_ERR_INVALID_ARGUMENT, "conformal time must stay positive");
    }
    const TileConfigEntry *cfg = config_for(lv->dtype, lv->tile_config);
    AXS_REQUIRE(cfg != nullptr, AXS_ERR_INVALID_ARGUMENT, "tile_config %d out of range (0..%d)", lv->tile_config,
                config_count(lv->dtype));
    SweepRunArgs r{lv, &g, bg, tau_i, t, dt, 1, 3, (cudaStream_t)stream, dst_state};
    return runner_for(lv, cfg)(r);
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
