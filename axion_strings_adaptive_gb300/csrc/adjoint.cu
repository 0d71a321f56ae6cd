// Hand-written discrete adjoint of the fused RK4 step, and the smooth
// string-core loss it is driven by.
//
// Forward step (see rk4_level.cu), with F_s(u) = lap u + [kappa_s - lambda_s/2 (|u|^2 - R_s^2)] u
// and stage coefficients s = 1 (t), 2 (t + h/2, stages 2 and 3), 4 (t + h):
//   u1 = psi, u2 = psi + h/2 Pi, u3 = u2 + h^2/4 F1(u1), u4 = psi + h Pi + h^2/2 F2(u2),
//   psi' = psi + h Pi + h^2/6 (F1 + F2 + F3),   Pi' = Pi + h/6 (F1 + 2 F2 + 2 F3 + F4),
//   F1 = F_1(u1), F2 = F_2(u2), F3 = F_2(u3), F4 = F_4(u4).
// Reverse step, given (psi'bar, Pi'bar):
//   F3bar = h^2/6 psi'bar + h/3 Pi'bar,   F4bar = h/6 Pi'bar,
//   u3bar = J_2(u3)^T F3bar,   u4bar = J_4(u4)^T F4bar,                  [adjoint sweep B]
//   F1bar = h^2/6 psi'bar + h/6 Pi'bar + h^2/4 u3bar,
//   F2bar = h^2/6 psi'bar + h/3 Pi'bar + h^2/2 u4bar,
//   u1bar = J_1(u1)^T F1bar,   u2bar = J_2(u2)^T F2bar + u3bar,          [adjoint sweep A]
//   psibar = psi'bar + u1bar + u2bar + u4bar,
//   Pibar  = Pi'bar + h psi'bar + h/2 u2bar + h u4bar,
// with J_s(u)^T a = lap a + kappa_s a - lambda_s/2 [(|u|^2 - R_s^2) a + 2 u (u . a)]
// (the periodic centred Laplacian is symmetric), and the lambda0 gradient
//   lambda0bar += sum_s sum_sites -(lambda_s/2)/lambda0 (|u_s|^2 - R_s^2) (u_s . F_sbar).
// u3 and u4 are recomputed by re-running forward sweep A on psi_n, Pi_n
// (it stores d3 = u3 - psi_n, d4 = u4 - psi_n).
// Each adjoint sweep is the same TMA-staged stencil pipeline as the forward
// sweeps (sweep.cuh); sweep B reads 4+6 and writes 8 components per site,
// sweep A reads 4+12 and writes 4.
#include <cmath>

#include "rk4_ops.cuh"

namespace axs {

int level_fill_ghosts(void *data, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g, int ncomp,
                      cudaStream_t st);
int make_level_map(CUtensorMap *map, const void *base, int32_t dtype, const LevelGeom &g, int ny, int nz,
                   uint32_t box_x, uint32_t box_y);

// Adjoint sweep B: stencil on (psi'bar, Pi'bar); pointwise (d3, d4) of the
// recomputed forward sweep A and psi_n, whose sums are the stage states
// u3 = psi_n + d3, u4 = psi_n + d4 (the forward sweep B forms them alike).
// Writes (F1bar, F2bar) with periodic copies and (u3bar, u4bar).
struct AdjointB {
    static constexpr int kPointwise = 6;
    static constexpr bool kLambdaGrad = true;
    static constexpr bool kComp = false;
    template <typename T, int V, bool HINT, typename PQ>
    __device__ static void apply(const SweepArgs<T> &a, const BoxGeom &b, const T (&lap)[4][V],
                                 const T (&ctr)[4][V], const PQ &pq, int64_t off, int x, int y, LamAcc<T> &lam,
                                 uint64_t pol)
    {
        T fo[4][V], uo[4][V];
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const T qb1 = ctr[0][v], qb2 = ctr[1][v], pb1 = ctr[2][v], pb2 = ctr[3][v];
            const T f3b1 = fma(a.h2_sixth, qb1, a.h_third * pb1), f3b2 = fma(a.h2_sixth, qb2, a.h_third * pb2);
            const T lf3b1 = fma(a.h2_sixth, lap[0][v], a.h_third * lap[2][v]);
            const T lf3b2 = fma(a.h2_sixth, lap[1][v], a.h_third * lap[3][v]);
            const T f4b1 = a.h_sixth * pb1, f4b2 = a.h_sixth * pb2;
            const T u31 = pq[4][v] + pq[0][v], u32 = pq[5][v] + pq[1][v];
            const T u41 = pq[4][v] + pq[2][v], u42 = pq[5][v] + pq[3][v];
            T u3b1, u3b2, u4b1, u4b2;
            rhs_adjoint_pair(a.c2, u31, u32, f3b1, f3b2, lf3b1, lf3b2, u3b1, u3b2);
            rhs_adjoint_pair(a.c4, u41, u42, f4b1, f4b2, a.h_sixth * lap[2][v], a.h_sixth * lap[3][v], u4b1, u4b2);
            const T base1 = fma(a.h2_sixth, qb1, a.h_sixth * pb1), base2 = fma(a.h2_sixth, qb2, a.h_sixth * pb2);
            fo[0][v] = fma(a.h2_quarter, u3b1, base1);  // F1bar
            fo[1][v] = fma(a.h2_quarter, u3b2, base2);
            fo[2][v] = fma(a.h2_half, u4b1, f3b1);      // F2bar = F3bar + h^2/2 u4bar
            fo[3][v] = fma(a.h2_half, u4b2, f3b2);
            uo[0][v] = u3b1;
            uo[1][v] = u3b2;
            uo[2][v] = u4b1;
            uo[3][v] = u4b2;
            // lambda0 gradient: per-site term in T, compensated sum in T (LamAcc)
            const T m3 = fma(u31, u31, fma(u32, u32, -a.c2.R2));
            const T m4 = fma(u41, u41, fma(u42, u42, -a.c4.R2));
            lam.add(-fma(a.c2.hlam * m3, fma(u31, f3b1, u32 * f3b2), a.c4.hlam * m4 * fma(u41, f4b1, u42 * f4b2)));
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
            store_with_copies<T, V, HINT>(a.out[c], off, x, y, b.nx, b.ny, b.js, fo[c], pol, b.periodic);
#pragma unroll
        for (int c = 0; c < 4; ++c) st_out<T, V, HINT>(a.out[4 + c] + off, uo[c], pol);
    }
};

// Adjoint sweep A: stencil on (F1bar, F2bar); pointwise (psi, Pi, u3bar, u4bar,
// psi'bar, Pi'bar). Writes (psibar, Pibar) with periodic copies.
struct AdjointA {
    static constexpr int kPointwise = 12;
    static constexpr bool kLambdaGrad = true;
    static constexpr bool kComp = false;
    template <typename T, int V, bool HINT, typename PQ>
    __device__ static void apply(const SweepArgs<T> &a, const BoxGeom &b, const T (&lap)[4][V],
                                 const T (&ctr)[4][V], const PQ &pq, int64_t off, int x, int y, LamAcc<T> &lam,
                                 uint64_t pol)
    {
        T o[4][V];
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const T p1 = pq[0][v], p2 = pq[1][v], q1 = pq[2][v], q2 = pq[3][v];
            const T u3b1 = pq[4][v], u3b2 = pq[5][v], u4b1 = pq[6][v], u4b2 = pq[7][v];
            const T qb1 = pq[8][v], qb2 = pq[9][v], pb1 = pq[10][v], pb2 = pq[11][v];
            const T f1b1 = ctr[0][v], f1b2 = ctr[1][v], f2b1 = ctr[2][v], f2b2 = ctr[3][v];
            const T u21 = fma(a.h_half, q1, p1), u22 = fma(a.h_half, q2, p2);
            T u1b1, u1b2, u2b1, u2b2;
            rhs_adjoint_pair(a.c1, p1, p2, f1b1, f1b2, lap[0][v], lap[1][v], u1b1, u1b2);
            rhs_adjoint_pair(a.c2, u21, u22, f2b1, f2b2, lap[2][v], lap[3][v], u2b1, u2b2);
            u2b1 += u3b1;
            u2b2 += u3b2;
            o[0][v] = qb1 + u1b1 + u2b1 + u4b1;
            o[1][v] = qb2 + u1b2 + u2b2 + u4b2;
            o[2][v] = fma(a.h, u4b1, fma(a.h_half, u2b1, fma(a.h, qb1, pb1)));
            o[3][v] = fma(a.h, u4b2, fma(a.h_half, u2b2, fma(a.h, qb2, pb2)));
            const T m1 = fma(p1, p1, fma(p2, p2, -a.c1.R2));
            const T m2 = fma(u21, u21, fma(u22, u22, -a.c2.R2));
            lam.add(-fma(a.c1.hlam * m1, fma(p1, f1b1, p2 * f1b2), a.c2.hlam * m2 * fma(u21, f2b1, u22 * f2b2)));
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
            store_with_copies<T, V, HINT>(a.out[c], off, x, y, b.nx, b.ny, b.js, o[c], pol, b.periodic);
    }
};

// Sum the per-block lambda0-gradient partials of both sweeps in a fixed order
// and add them to the caller's accumulator.
__global__ void lambda_bar_finalize_kernel(const double *__restrict__ part, int n, double *__restrict__ acc)
{
    __shared__ double s[256];
    double x = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) x += part[i];
    s[threadIdx.x] = x;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *acc += s[0];
}

// ----------------------------------------------------------------------------
// Smooth string-core loss at the final time (its gradient seeds the adjoint):
//   L = sum_cells exp(-|phi|^2 / w) + (1/N) sum_cells (theta'/R)^2,  phi = psi/R,
// the second term being the unscreened axion kinetic energy density average
// (Energy.hpp:90-97: 1/2 (sqrt(2) theta'/R)^2, theta' = (psi1 Pi2 - Pi1 psi2)/|psi|^2).
template <typename T>
__global__ void string_core_loss_kernel(const T *__restrict__ st, T *__restrict__ grad, LevelGeom g, int nx, int ny,
                                        int nz, double inv_wR2, double inv_NR2, double *__restrict__ partials)
{
    const int64_t n = (int64_t)nx * ny * nz;
    double acc = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(q % nx), y = (int)((q / nx) % ny), z = (int)(q / ((int64_t)nx * ny));
        const int64_t o = (x + g.ox) + (int64_t)(y + g.oy) * g.js + (int64_t)z * g.ks;
        const double p1 = st[o], p2 = st[g.cs + o], q1 = st[2 * g.cs + o], q2 = st[3 * g.cs + o];
        const double psq = p1 * p1 + p2 * p2;
        const double ea = exp(-psq * inv_wR2);
        double gp1 = -2.0 * inv_wR2 * ea * p1, gp2 = -2.0 * inv_wR2 * ea * p2, gq1 = 0.0, gq2 = 0.0;
        double loss = ea;
        if (psq > 0.0) {
            const double ip = 1.0 / psq;
            const double c = p1 * q2 - q1 * p2;
            const double th = c * ip;
            loss += th * th * inv_NR2;
            const double k = 2.0 * th * inv_NR2;
            gp1 += k * (q2 * ip - 2.0 * p1 * c * ip * ip);
            gp2 += k * (-q1 * ip - 2.0 * p2 * c * ip * ip);
            gq1 += k * (-p2 * ip);
            gq2 += k * (p1 * ip);
        }
        acc += loss;
        if (grad) {
            grad[o] = (T)gp1;
            grad[g.cs + o] = (T)gp2;
            grad[2 * g.cs + o] = (T)gq1;
            grad[3 * g.cs + o] = (T)gq2;
        }
    }
    __shared__ double s[256];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = s[0];
}

__global__ void sum_partials_kernel(const double *__restrict__ part, int n, double *__restrict__ out)
{
    __shared__ double s[256];
    double x = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) x += part[i];
    s[threadIdx.x] = x;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s[0];
}

// ----------------------------------------------------------------------------
// Adjoint tiling: one configuration per dtype (V = 1 keeps the 12 pointwise
// components of sweep A in registers without spilling).
constexpr int kAdjMaxGridPerSm = 4;

template <typename T> struct AdjointRunner {
    using LB = SweepLauncher<T, 1, 32, 8, 8, 2, AdjointB>;
    using LA = SweepLauncher<T, 1, 32, 8, 8, 2, AdjointA>;

    static int run(const axs_level *lv, const LevelGeom &g, T *abar, T *adj, double *lam_part, int lam_slots,
                   const axs_background &bg, double tau_i, double t, double dt, double *lam_acc, cudaStream_t st)
    {
        SweepArgs<T> a{};
        int grid_b = 0, grid_a = 0;
        int rc = LB::plan(a, lv->nx, lv->ny, lv->nz, grid_b);
        if (rc) return rc;
        SweepArgs<T> pa = a;
        if ((rc = LA::plan(pa, lv->nx, lv->ny, lv->nz, grid_a))) return rc;
        AXS_REQUIRE(grid_a + grid_b <= lam_slots, AXS_ERR_WORKSPACE, "adjoint scratch too small for %d blocks",
                    grid_a + grid_b);
        // step constants (shared with the forward sweeps)
        a.js = g.js;
        a.ks = g.ks;
        a.cs = g.cs;
        a.ox = g.ox;
        fill_step_constants(a, lv->dx, dt);
        a.inv_lambda0 = 1.0 / bg.lambda_scale;
        a.c1 = stage_coef<T>(bg, tau_i + t);
        a.c2 = stage_coef<T>(bg, tau_i + t + 0.5 * dt);
        a.c4 = stage_coef<T>(bg, tau_i + t + dt);
        a.status = reinterpret_cast<unsigned *>(static_cast<char *>(lv->work) + 8 * g.cs * sizeof(T));
        const T *state = static_cast<const T *>(lv->state);
        const T *work = static_cast<const T *>(lv->work);
        T *fbar = adj, *ubar = adj + 4 * g.cs;

        CUtensorMap map_abar, map_fbar;
        if ((rc = make_level_map(&map_abar, abar, lv->dtype, g, lv->ny, lv->nz, LB::box_x(), LB::box_y()))) return rc;
        if ((rc = make_level_map(&map_fbar, fbar, lv->dtype, g, lv->ny, lv->nz, LA::box_x(), LA::box_y()))) return rc;

        SweepArgs<T> b = a;  // adjoint sweep B
        for (int c = 0; c < 4; ++c) b.pt[c] = work + c * g.cs;  // d3, d4 from forward sweep A
        for (int c = 0; c < 2; ++c) b.pt[4 + c] = state + c * g.cs;  // psi_n
        for (int c = 0; c < 4; ++c) b.out[c] = fbar + c * g.cs;
        for (int c = 0; c < 4; ++c) b.out[4 + c] = ubar + c * g.cs;
        b.lam_partial = lam_part;
        if ((rc = LB::launch(map_abar, b, grid_b, st))) return rc;

        SweepArgs<T> s = a;  // adjoint sweep A
        s.n_items = pa.n_items;
        s.zchunk = pa.zchunk;
        for (int c = 0; c < 4; ++c) s.pt[c] = state + c * g.cs;
        for (int c = 0; c < 4; ++c) s.pt[4 + c] = ubar + c * g.cs;
        for (int c = 0; c < 4; ++c) s.pt[8 + c] = abar + c * g.cs;
        for (int c = 0; c < 4; ++c) s.out[c] = abar + c * g.cs;
        s.lam_partial = lam_part + grid_b;
        if ((rc = LA::launch(map_fbar, s, grid_a, st))) return rc;
        lambda_bar_finalize_kernel<<<1, 256, 0, st>>>(lam_part, grid_a + grid_b, lam_acc);
        return launch_status("lambda0 gradient finalize");
    }
};

static int lam_slots_for()
{
    const int sms = device_sm_count();
    return (sms > 0 ? sms : 148) * kAdjMaxGridPerSm * 2;
}

}  // namespace axs

using namespace axs;

extern "C" {

int axs_level_adjoint_work_bytes(int32_t dtype, int32_t nx, int32_t ny, int32_t nz, int64_t *bytes)
{
    AXS_REQUIRE(bytes != nullptr, AXS_ERR_INVALID_ARGUMENT, "null output");
    LevelGeom g;
    int rc = level_geom(dtype, nx, ny, nz, g);
    if (rc) return rc;
    *bytes = 8 * g.cs * (int64_t)dtype_size(dtype) + (int64_t)lam_slots_for() * (int64_t)sizeof(double);
    return AXS_OK;
}

int axs_level_rk4_adjoint_step(const axs_level *lv, void *abar, void *adj_work, int64_t adj_work_bytes,
                               const axs_background *bg, double tau_i, double t, double dt, double *lambda0_bar,
                               void *stream)
{
    AXS_REQUIRE(lv != nullptr && abar != nullptr && adj_work != nullptr && bg != nullptr && lambda0_bar != nullptr,
                AXS_ERR_INVALID_ARGUMENT, "null argument");
    AXS_REQUIRE(lv->state && lv->work, AXS_ERR_INVALID_ARGUMENT, "level state/work is null");
    LevelGeom g;
    int rc = level_geom(lv->dtype, lv->nx, lv->ny, lv->nz, g);
    if (rc) return rc;
    AXS_REQUIRE(((uintptr_t)abar % 128) == 0 && ((uintptr_t)adj_work % 128) == 0, AXS_ERR_ALIGNMENT,
                "adjoint buffers must be 128-byte aligned");
    AXS_REQUIRE(std::isfinite(dt) && dt > 0.0, AXS_ERR_INVALID_ARGUMENT, "dt must be positive and finite");
    AXS_REQUIRE(bg->lambda_scale != 0.0, AXS_ERR_INVALID_ARGUMENT, "lambda_scale must be nonzero");
    int64_t need = 0;
    axs_level_adjoint_work_bytes(lv->dtype, lv->nx, lv->ny, lv->nz, &need);
    AXS_REQUIRE(adj_work_bytes >= need, AXS_ERR_WORKSPACE, "adjoint workspace too small (%lld < %lld bytes)",
                (long long)adj_work_bytes, (long long)need);
    cudaStream_t st = (cudaStream_t)stream;
    // recompute the stage fields u3, u4 of this step into lv->work
    rc = axs_level_rk4_sweep(lv, bg, tau_i, t, dt, 0, stream);
    if (rc) return rc;
    const size_t es = dtype_size(lv->dtype);
    double *lam_part = reinterpret_cast<double *>(static_cast<char *>(adj_work) + 8 * g.cs * es);
    if (lv->dtype == AXS_F32)
        return AdjointRunner<float>::run(lv, g, static_cast<float *>(abar), static_cast<float *>(adj_work), lam_part,
                                         lam_slots_for(), *bg, tau_i, t, dt, lambda0_bar, st);
    return AdjointRunner<double>::run(lv, g, static_cast<double *>(abar), static_cast<double *>(adj_work), lam_part,
                                      lam_slots_for(), *bg, tau_i, t, dt, lambda0_bar, st);
}

int axs_level_string_core_loss(const axs_level *lv, double R, double width, double *loss_dev, void *grad,
                               void *scratch, int64_t scratch_bytes, void *stream)
{
    AXS_REQUIRE(lv != nullptr && lv->state != nullptr && loss_dev != nullptr && scratch != nullptr,
                AXS_ERR_INVALID_ARGUMENT, "null argument");
    AXS_REQUIRE(R > 0.0 && width > 0.0, AXS_ERR_INVALID_ARGUMENT, "R and width must be positive");
    LevelGeom g;
    int rc = level_geom(lv->dtype, lv->nx, lv->ny, lv->nz, g);
    if (rc) return rc;
    const int sms = device_sm_count();
    const int grid = (sms > 0 ? sms : 148) * 4;
    AXS_REQUIRE(scratch_bytes >= (int64_t)grid * 8, AXS_ERR_WORKSPACE, "loss scratch needs %d bytes", grid * 8);
    cudaStream_t st = (cudaStream_t)stream;
    const double inv_wR2 = 1.0 / (width * R * R);
    const double inv_NR2 = 1.0 / ((double)lv->nx * lv->ny * lv->nz * R * R);
    double *part = static_cast<double *>(scratch);
    if (lv->dtype == AXS_F32)
        string_core_loss_kernel<float><<<grid, 256, 0, st>>>(static_cast<const float *>(lv->state),
                                                             static_cast<float *>(grad), g, lv->nx, lv->ny, lv->nz,
                                                             inv_wR2, inv_NR2, part);
    else
        string_core_loss_kernel<double><<<grid, 256, 0, st>>>(static_cast<const double *>(lv->state),
                                                              static_cast<double *>(grad), g, lv->nx, lv->ny, lv->nz,
                                                              inv_wR2, inv_NR2, part);
    if ((rc = launch_status("string core loss"))) return rc;
    sum_partials_kernel<<<1, 256, 0, st>>>(part, grid, loss_dev);
    if ((rc = launch_status("loss sum"))) return rc;
    if (grad) return level_fill_ghosts(grad, lv->dtype, lv->nx, lv->ny, lv->nz, g, 4, st);
    return AXS_OK;
}

}  // extern "C"
