// Drop-in kernels on AMReX-layout FABs: the per-stage RHS that replaces the
// body of AxionStringsLevel::specific_eval_rhs, the periodic ghost fill, the
// RK stage combinations, and copies between FABs and the fused-RK4 level
// layout.
#include <algorithm>
#include "axs_internal.cuh"

namespace axs {

// Offset of cell (i,j,k) of component 0 in a FAB (i etc. may be negative ghosts).
__host__ __device__ __forceinline__ int64_t fab_off(const axs_fab &f, int i, int j, int k)
{
    return (int64_t)(i + f.ng) + (int64_t)(j + f.ng) * f.jstride + (int64_t)(k + f.ng) * f.kstride;
}

// The kernels below walk x rows one warp per row: a row's (j, k, component)
// comes from two 32-bit divisions per row, and the lanes read and write
// consecutive x. Warps take rows with a grid stride.
__device__ __forceinline__ int row_warp() { return (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); }
__device__ __forceinline__ int row_warps() { return (int)((gridDim.x * blockDim.x) >> 5); }

struct RowIdx {
    int j, k, c;
};

// Row r of `ny` rows per plane and `nz` planes per component.
__device__ __forceinline__ RowIdx row_index(int r, int ny, int nz)
{
    RowIdx q;
    const int plane = r / ny;
    q.j = r - plane * ny;
    q.c = plane / nz;
    q.k = plane - q.c * nz;
    return q;
}

// ---------------------------------------------------------------- RHS
// AxionStringsRHS<FourthOrderDerivatives>::operator() (AxionStringsRHS.impl.hpp:25-60).
// FP64: evaluated with the reference's expression order and explicit
// round-to-nearest intrinsics (no FMA contraction), so it reproduces the
// host evaluation of the same expressions bit for bit. Laplacian weights are
// GRTeclyn's centred 4th-order diff2 (1/12, 4/3, 5/2) * 1/dx^2.
__device__ __forceinline__ double diff2_exact(const double *__restrict__ p, int64_t s, double one_over_dx2)
{
    const double wf = 8.33333333333333333333e-2;
    const double wn = 1.33333333333333333333e+0;
    const double wl = 2.50000000000000000000e+0;
    double r = __dmul_rn(-wf, __ldg(p - 2 * s));
    r = __dadd_rn(r, __dmul_rn(wn, __ldg(p - s)));
    r = __dsub_rn(r, __dmul_rn(wl, __ldg(p)));
    r = __dadd_rn(r, __dmul_rn(wn, __ldg(p + s)));
    r = __dsub_rn(r, __dmul_rn(wf, __ldg(p + 2 * s)));
    return __dmul_rn(r, one_over_dx2);
}

__global__ void eval_rhs_f64_kernel(const axs_fab s, const axs_fab r, double one_over_dx2, double kappa,
                                    double lambda, double R2)
{
    const double *__restrict__ sp = static_cast<const double *>(s.data);
    double *__restrict__ rp = static_cast<double *>(r.data);
    const int rows = s.ny * s.nz, lane = threadIdx.x & 31;
    const int64_t st[3] = {1, s.jstride, s.kstride};
    for (int row = row_warp(); row < rows; row += row_warps()) {
        const RowIdx q = row_index(row, s.ny, s.nz);
        const int64_t o0 = fab_off(s, 0, q.j, q.k), r0 = fab_off(r, 0, q.j, q.k);
        for (int i = lane; i < s.nx; i += 32) {
            const int64_t o = o0 + i;
            double lap1 = 0.0, lap2 = 0.0;
#pragma unroll
            for (int d = 0; d < 3; ++d) lap1 = __dadd_rn(lap1, diff2_exact(sp + o, st[d], one_over_dx2));
#pragma unroll
            for (int d = 0; d < 3; ++d) lap2 = __dadd_rn(lap2, diff2_exact(sp + s.cstride + o, st[d], one_over_dx2));
            const double psi1 = sp[o], psi2 = sp[s.cstride + o];
            const double dsq = __dsub_rn(__dadd_rn(__dmul_rn(psi1, psi1), __dmul_rn(psi2, psi2)), R2);
            const double pc = __dmul_rn(__dmul_rn(0.5, lambda), dsq);
            const int64_t ro = r0 + i;
            rp[ro] = sp[2 * s.cstride + o];
            rp[r.cstride + ro] = sp[3 * s.cstride + o];
            rp[2 * r.cstride + ro] = __dsub_rn(__dadd_rn(lap1, __dmul_rn(kappa, psi1)), __dmul_rn(pc, psi1));
            rp[3 * r.cstride + ro] = __dsub_rn(__dadd_rn(lap2, __dmul_rn(kappa, psi2)), __dmul_rn(pc, psi2));
        }
    }
}

// FP32 (the reference's default PRECISION=FLOAT build): single-precision
// arithmetic throughout, contraction allowed; the Laplacian sums the x, y and
// z second differences in that order, each (-wf, wn, -wl, wn, -wf) . f / dx^2.
// Marched along z: a block owns a 32 x TY column of cells and ZC planes of it.
// Plane p's psi1, psi2 over the tile plus a 2-cell x/y halo, and Pi1, Pi2 over
// the tile, are copied by cp.async into a (D + 5)-slot shared-memory ring, D
// planes ahead of the plane the block computes: every stencil operand then
// comes from shared memory, each staged value is read from global memory once
// per block, and a thread keeps about 5 D copies in flight.
// W16: FABs whose psi tile rows start 16-byte aligned (ng = 2 mod 4, strides
// multiples of 4 elements, a 16-byte aligned base) and whose extents are
// multiples of the block tile (nx of 32, ny of TY): the tile's rows are copied
// in 16-byte pieces (9 per 36-column row), Pi over the same 36-column rows, and
// no piece leaves the ghost region, so no zero-fill is needed.
template <int TY, int ZC, int D, bool W16>
__global__ void __launch_bounds__(32 * TY) eval_rhs_f32_zmarch_kernel(const axs_fab s, const axs_fab r,
                                                                      float one_over_dx2, float kappa, float lambda,
                                                                      float R2)
{
    constexpr int SX = 36, SY = TY + 4, PSI = SX * SY, NT = 32 * TY;
    constexpr int PI = W16 ? TY * SX : NT;  // one Pi component of a slot
    constexpr int SLOT = 2 * PSI + 2 * PI, NSLOT = D + 5;
    constexpr int NPS = W16 ? (2 * SY * 9 + 2 * TY * 9 + NT - 1) / NT : (2 * PSI + NT - 1) / NT;
    static_assert(!W16 || (SLOT % 4 == 0 && PSI % 4 == 0 && PI % 4 == 0), "16-byte pieces land 16-byte aligned");
    __shared__ __align__(16) float sh[NSLOT * SLOT];
    const float *__restrict__ sp = static_cast<const float *>(s.data);
    float *__restrict__ rp = static_cast<float *>(r.data);
    const float wf = 8.33333333333333333333e-2f, wn = 1.33333333333333333333e+0f, wl = 2.5f;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * TY, z0 = blockIdx.z * ZC;
    const int z1 = min(z0 + ZC, s.nz);
    const int i = x0 + tx, j = y0 + ty;
    const bool in = i < s.nx && j < s.ny;
    const int64_t o0 = fab_off(s, in ? i : 0, in ? j : 0, 0), ro0 = fab_off(r, in ? i : 0, in ? j : 0, 0);
    // This thread's staging tasks: plane-0 global offset, shared offset within a
    // slot, and whether the task copies (W16: 16-byte pieces of psi rows, then of
    // Pi rows; else psi cells, zero-filled outside the FAB's 2 ghost layers).
    int64_t st_off[NPS];
    int st_sh[NPS];
    bool st_ok[NPS];
#pragma unroll
    for (int q = 0; q < NPS; ++q) {
        const int e = tid + q * NT;
        if constexpr (W16) {
            const int npsi = 2 * SY * 9, e2 = e - npsi;
            const bool is_psi = e < npsi;
            const int rows = is_psi ? SY : TY, ee = is_psi ? e : e2;
            const int c = ee / (rows * 9), rem = ee - c * rows * 9, row = rem / 9, k = rem - row * 9;
            st_ok[q] = is_psi || e2 < 2 * TY * 9;
            const int gj = is_psi ? y0 - 2 + row : y0 + row;
            st_off[q] = st_ok[q] ? (is_psi ? c : 2 + c) * s.cstride + fab_off(s, x0 - 2 + 4 * k, gj, 0) : 0;
            st_sh[q] = (is_psi ? c * PSI : 2 * PSI + c * PI) + row * SX + 4 * k;
        } else {
            const int c = e >= PSI, rem = e - c * PSI, yy = rem / SX, xx = rem - yy * SX;
            const int gi = x0 - 2 + xx, gj = y0 - 2 + yy;
            st_ok[q] = e < 2 * PSI && gi < s.nx + 2 && gj < s.ny + 2;
            st_off[q] = st_ok[q] ? c * s.cstride + fab_off(s, gi, gj, 0) : 0;
            st_sh[q] = e;
        }
    }
    auto slot = [&](int p) { return sh + ((p - z0 + 2) % NSLOT) * SLOT; };
    auto issue = [&](int p) {
        if (p > z1 + 1) return;  // beyond the last plane a computed cell reads
        float *dst = slot(p);
        const int64_t po = (int64_t)p * s.kstride;
        if constexpr (W16) {
            // psi pieces for every staged plane; Pi pieces only for the computed planes
#pragma unroll
            for (int q = 0; q < NPS; ++q) {
                const bool pi_piece = st_sh[q] >= 2 * PSI;
                if (st_ok[q] && (!pi_piece || (p >= z0 && p < z1))) {
                    const unsigned d = (unsigned)__cvta_generic_to_shared(dst + st_sh[q]);
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(sp + st_off[q] + po)
                                 : "memory");
                }
            }
        } else {
#pragma unroll
            for (int q = 0; q < NPS; ++q)
                if (tid + q * NT < 2 * PSI) cp_async_elem(dst + st_sh[q], sp + st_off[q] + po, st_ok[q], sp);
            if (p >= z0 && p < z1) {
                cp_async_elem(dst + 2 * PSI + tid, sp + 2 * s.cstride + o0 + po, in, sp);
                cp_async_elem(dst + 2 * PSI + PI + tid, sp + 3 * s.cstride + o0 + po, in, sp);
            }
        }
    };
    for (int p = z0 - 2; p <= z0 + 1 + D; ++p) {
        issue(p);
        cp_async_commit();
    }
    const int c0 = (ty + 2) * SX + tx + 2;                    // this thread's cell in a plane's psi tile
    const int pi0 = 2 * PSI + (W16 ? ty * SX + tx + 2 : tid);  // ... and in its Pi tile
    for (int z = z0; z < z1; ++z) {
        cp_async_wait<D - 1>();  // planes up to z + 2 have landed (this thread's copies)
        __syncthreads();         // ... and everyone's; the slot of plane z - 3 is free
        issue(z + 2 + D);
        cp_async_commit();
        if (in) {
            const float *t = slot(z);
            const float *zm2 = slot(z - 2), *zm1 = slot(z - 1), *zp1 = slot(z + 1), *zp2 = slot(z + 2);
            float lap[2];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const int b = c * PSI + c0;
                float acc = 0.f;
                acc += (-wf * t[b - 2] + wn * t[b - 1] - wl * t[b] + wn * t[b + 1] - wf * t[b + 2]) * one_over_dx2;
                acc += (-wf * t[b - 2 * SX] + wn * t[b - SX] - wl * t[b] + wn * t[b + SX] - wf * t[b + 2 * SX]) *
                       one_over_dx2;
                acc += (-wf * zm2[b] + wn * zm1[b] - wl * t[b] + wn * zp1[b] - wf * zp2[b]) * one_over_dx2;
                lap[c] = acc;
            }
            const int64_t ro = ro0 + (int64_t)z * r.kstride;
            const float psi1 = t[c0], psi2 = t[PSI + c0];
            const float pc = 0.5f * lambda * (psi1 * psi1 + psi2 * psi2 - R2);
            rp[ro] = t[pi0];
            rp[r.cstride + ro] = t[pi0 + PI];
            rp[2 * r.cstride + ro] = lap[0] + kappa * psi1 - pc * psi1;
            rp[3 * r.cstride + ro] = lap[1] + kappa * psi2 - pc * psi2;
        }
    }
}

// ---------------------------------------------------------------- ghost fill
// Periodic images into the ghost cells only (ng <= each extent, so one wrap
// reaches the valid box and no ghost reads another ghost). Per component
// (blockIdx.y): the full ghost rows -- all rows of the 2 ng z ghost planes when
// `with_z`, and the 2 ng y ghost rows of every valid plane -- one warp per row,
// then the 2 ng x ghosts of each valid row one thread per cell. With with_z = 0
// the z ghost planes are left alone (a z slab of a larger periodic box: they
// come from the neighbouring slabs).
__device__ __forceinline__ int wrap_once(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

template <typename T>
__global__ void fill_periodic_kernel(const axs_fab f, int with_z)
{
    T *p = static_cast<T *>(f.data) + blockIdx.y * f.cstride;
    const int ng = f.ng, gy = f.ny + 2 * ng, lane = threadIdx.x & 31;
    const int zrows = with_z ? 2 * ng * gy : 0, rows = zrows + f.nz * 2 * ng;
    for (int r = row_warp(); r < rows; r += row_warps()) {
        int j, k;
        if (r < zrows) {
            const int kz = r / gy;
            j = r - kz * gy - ng;
            k = kz < ng ? kz - ng : f.nz + kz - ng;
        } else {
            const int b = r - zrows, g = b % (2 * ng);
            k = b / (2 * ng);
            j = g < ng ? g - ng : f.ny + g - ng;
        }
        T *dst = p + fab_off(f, 0, j, k);
        const T *src = p + fab_off(f, 0, wrap_once(j, f.ny), wrap_once(k, f.nz));
        for (int x = lane - ng; x < f.nx + ng; x += 32) dst[x] = src[wrap_once(x, f.nx)];
    }
    const int cells = f.ny * f.nz * 2 * ng;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cells; e += gridDim.x * blockDim.x) {
        const int row = e / (2 * ng), g = e - row * 2 * ng;
        const int k = row / f.ny, j = row - k * f.ny;
        const int x = g < ng ? g - ng : f.nx + g - ng;
        T *q = p + fab_off(f, 0, j, k);
        q[x] = q[wrap_once(x, f.nx)];
    }
}

// Whole padded planes z0 .. z0 + np - 1 (ghost planes allowed: -ng <= z) of all
// components, between the FAB and a contiguous (ncomp, np, ny+2ng, nx+2ng) buffer.
template <typename T>
__global__ void copy_z_planes_kernel(const axs_fab f, int z0, int np, T *buf, int to_buf)
{
    const int gx = f.nx + 2 * f.ng, gy = f.ny + 2 * f.ng, lane = threadIdx.x & 31;
    const int rows = gy * np * f.ncomp;
    for (int r = row_warp(); r < rows; r += row_warps()) {
        const RowIdx q = row_index(r, gy, np);
        T *e = static_cast<T *>(f.data) + q.c * f.cstride + fab_off(f, -f.ng, q.j - f.ng, z0 + q.k);
        T *b = buf + (int64_t)r * gx;
        for (int x = lane; x < gx; x += 32) {
            if (to_buf)
                b[x] = e[x];
            else
                e[x] = b[x];
        }
    }
}

// ---------------------------------------------------------------- stage combinations
// Evaluated with explicit round-to-nearest operations in the host's
// expression order (no contraction), so the per-stage drop-in path reproduces
// a CPU evaluation of the same RK4 bit for bit.
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float rn_div(float a, float b) { return __fdiv_rn(a, b); }

template <typename T>
__global__ void lincomb_kernel(const axs_fab d, const axs_fab x, T b, const axs_fab y, int ncomp)
{
    const int rows = d.ny * d.nz * ncomp, lane = threadIdx.x & 31;
    for (int r = row_warp(); r < rows; r += row_warps()) {
        const RowIdx q = row_index(r, d.ny, d.nz);
        T *dr = static_cast<T *>(d.data) + q.c * d.cstride + fab_off(d, 0, q.j, q.k);
        const T *xr = static_cast<const T *>(x.data) + q.c * x.cstride + fab_off(x, 0, q.j, q.k);
        const T *yr = static_cast<const T *>(y.data) + q.c * y.cstride + fab_off(y, 0, q.j, q.k);
        for (int i0 = lane; i0 < d.nx; i0 += 128) {
            T xv[4], yv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i0 + 32 * u < d.nx) xv[u] = xr[i0 + 32 * u], yv[u] = yr[i0 + 32 * u];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i0 + 32 * u < d.nx) dr[i0 + 32 * u] = rn_add(xv[u], rn_mul(b, yv[u]));
        }
    }
}

template <typename T>
__global__ void rk4_combine_kernel(const axs_fab d, const axs_fab u, const axs_fab k1, const axs_fab k2,
                                   const axs_fab k3, const axs_fab k4, T h6, int ncomp)
{
    const int rows = d.ny * d.nz * ncomp, lane = threadIdx.x & 31;
    for (int r = row_warp(); r < rows; r += row_warps()) {
        const RowIdx q = row_index(r, d.ny, d.nz);
        auto row = [&](const axs_fab &f) {
            return static_cast<const T *>(f.data) + q.c * f.cstride + fab_off(f, 0, q.j, q.k);
        };
        const T *ur = row(u), *a = row(k1), *b = row(k2), *c = row(k3), *e = row(k4);
        T *dr = static_cast<T *>(d.data) + q.c * d.cstride + fab_off(d, 0, q.j, q.k);
        for (int i0 = lane; i0 < d.nx; i0 += 64) {
            T v[2][5];
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                const int i = i0 + 32 * w;
                if (i < d.nx) v[w][0] = a[i], v[w][1] = b[i], v[w][2] = c[i], v[w][3] = e[i], v[w][4] = ur[i];
            }
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                const int i = i0 + 32 * w;
                if (i < d.nx) {
                    const T sum = rn_add(rn_add(rn_add(v[w][0], rn_mul(T(2), v[w][1])), rn_mul(T(2), v[w][2])), v[w][3]);
                    dr[i] = rn_add(v[w][4], rn_mul(h6, sum));
                }
            }
        }
    }
}

// ---------------------------------------------------------------- level <-> FAB
// Level layout: (x + ox) + (y + oy)*js + z*ks + c*cs (see axs_level_layout).
template <typename T>
__global__ void level_from_fab_kernel(T *lv, LevelGeom g, const axs_fab f, int to_level)
{
    T *fp = static_cast<T *>(f.data);
    const int64_t nc = (int64_t)f.nx * f.ny * f.nz;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nc * 4; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t cell = q % nc;
        const int c = (int)(q / nc);
        const int i = (int)(cell % f.nx), j = (int)((cell / f.nx) % f.ny), k = (int)(cell / ((int64_t)f.nx * f.ny));
        const int64_t lo = c * g.cs + (i + g.ox) + (int64_t)(j + g.oy) * g.js + (int64_t)k * g.ks;
        const int64_t fo = c * f.cstride + fab_off(f, i, j, k);
        if (to_level)
            lv[lo] = fp[fo];
        else
            fp[fo] = lv[lo];
    }
}

// Periodic copies in the 8-column x and 2-row y padding of `ncomp` level
// components (corners included).
template <typename T>
__global__ void level_fill_ghosts_kernel(T *lv, int nx, int ny, int nz, LevelGeom g, int ncomp)
{
    const int px = nx + 16, py = ny + 4;  // 8 padding columns either side, as the sweeps keep them
    const int64_t n = (int64_t)px * py * nz * ncomp;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(q % px) - 8;
        const int y = (int)((q / px) % py) - 2;
        const int z = (int)((q / ((int64_t)px * py)) % nz);
        const int c = (int)(q / ((int64_t)px * py * nz));
        if (x >= 0 && x < nx && y >= 0 && y < ny) continue;
        const int xx = ((x % nx) + nx) % nx, yy = ((y % ny) + ny) % ny;
        T *base = lv + c * g.cs + (int64_t)z * g.ks;
        base[(x + g.ox) + (int64_t)(y + g.oy) * g.js] = base[(xx + g.ox) + (int64_t)(yy + g.oy) * g.js];
    }
}

// Contiguous (4, nz, ny, nx) array -> level layout: valid cells and the
// periodic padding (8 columns either side in x, 2 rows in y, corners included)
// in one pass. One block per padded row; consecutive threads take consecutive
// x, so reads and writes are coalesced.
template <typename T>
__global__ void level_scatter_kernel(T *__restrict__ lv, const T *__restrict__ src, int nx, int ny, int nz,
                                     LevelGeom g)
{
    const int64_t rows = (int64_t)(ny + 4) * nz * 4;
    for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const int y = (int)(r % (ny + 4)) - 2;
        const int64_t zc = r / (ny + 4);  // z + nz c
        const int z = (int)(zc % nz), c = (int)(zc / nz);
        const int ys = ((y % ny) + ny) % ny;
        const T *s = src + ((int64_t)c * nz + z) * ny * nx + (int64_t)ys * nx;
        T *d = lv + c * g.cs + (int64_t)z * g.ks + (int64_t)(y + g.oy) * g.js + g.ox;
        if (nx >= 8) {
            for (int x = (int)threadIdx.x - 8; x < nx + 8; x += blockDim.x) d[x] = s[x < 0 ? x + nx : (x >= nx ? x - nx : x)];
        } else {
            for (int x = (int)threadIdx.x - 8; x < nx + 8; x += blockDim.x) d[x] = s[((x % nx) + nx) % nx];
        }
    }
}

// Level layout -> contiguous (4, nz, ny, nx) array, valid cells only.
template <typename T>
__global__ void level_gather_kernel(const T *__restrict__ lv, T *__restrict__ dst, int nx, int ny, int nz,
                                    LevelGeom g)
{
    const int64_t rows = (int64_t)ny * nz * 4;
    for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const int y = (int)(r % ny);
        const int64_t zc = r / ny;
        const int z = (int)(zc % nz), c = (int)(zc / nz);
        const T *s = lv + c * g.cs + (int64_t)z * g.ks + (int64_t)(y + g.oy) * g.js + g.ox;
        T *d = dst + r * nx;
        for (int x = threadIdx.x; x < nx; x += blockDim.x) d[x] = s[x];
    }
}

// Pre-evolution -> main handoff (AxionStringsLevel.cpp:2027-2132) on the valid
// cells of a level, in the field precision with the reference's operation
// order: kappa = R_main/R_pre, common = R_main' - kappa^2 R_pre',
// psi <- kappa psi, Pi <- kappa^2 Pi + (psi/R_pre) common.
template <typename T>
__global__ void level_handoff_kernel(T *lv, int nx, int ny, int nz, LevelGeom g, T R_pre, T R_pre_prime, T R_main,
                                     T R_main_prime)
{
    const T kappa = rn_div(R_main, R_pre);
    const T kk = rn_mul(kappa, kappa);
    const T common = rn_sub(R_main_prime, rn_mul(kk, R_pre_prime));
    const int64_t n = (int64_t)nx * ny * nz;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(q % nx), y = (int)((q / nx) % ny), z = (int)(q / ((int64_t)nx * ny));
        const int64_t o = (x + g.ox) + (int64_t)(y + g.oy) * g.js + (int64_t)z * g.ks;
        const T p1 = lv[o], p2 = lv[g.cs + o], q1 = lv[2 * g.cs + o], q2 = lv[3 * g.cs + o];
        lv[o] = rn_mul(kappa, p1);
        lv[g.cs + o] = rn_mul(kappa, p2);
        lv[2 * g.cs + o] = rn_add(rn_mul(kk, q1), rn_mul(rn_div(p1, R_pre), common));
        lv[3 * g.cs + o] = rn_add(rn_mul(kk, q2), rn_mul(rn_div(p2, R_pre), common));
    }
}

// Cells (valid region from `base`, strides js, ks, cs) with a non-finite
// component, summed per warp and added to *count with one atomic per warp.
template <typename T>
__global__ void count_nonfinite_kernel(const T *__restrict__ base, int nx, int ny, int nz, int64_t js, int64_t ks,
                                       int64_t cs, unsigned long long *__restrict__ count)
{
    const int64_t n = (int64_t)nx * ny * nz;
    unsigned long long c = 0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(q % nx), y = (int)((q / nx) % ny), z = (int)(q / ((int64_t)nx * ny));
        const T *p = base + x + (int64_t)y * js + (int64_t)z * ks;
        const bool bad = !isfinite(p[0]) || !isfinite(p[cs]) || !isfinite(p[2 * cs]) || !isfinite(p[3 * cs]);
        c += bad ? 1u : 0u;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

static int grid_for(int64_t n)
{
    const int sms = device_sm_count();
    int64_t g = (n + 255) / 256;
    const int64_t cap = (int64_t)(sms > 0 ? sms : 148) * 16;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

// Blocks of 256 threads (8 row-walking warps) for `rows` rows: up to 8 blocks
// per SM, grid-stride beyond that.
static int grid_rows(int64_t rows)
{
    const int sms = device_sm_count();
    int64_t g = (rows + 7) / 8;
    const int64_t cap = (int64_t)(sms > 0 ? sms : 148) * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

// The row-walking kernels index rows and ghost cells in 32 bits.
static int rows_fit(const axs_fab *f, const char *what)
{
    const int64_t ry = f->ny + 2LL * f->ng, rz = f->nz + 2LL * f->ng;
    AXS_REQUIRE(ry * rz * f->ncomp * (2LL * f->ng + 1) < (1LL << 31), AXS_ERR_UNSUPPORTED,
                "%s: %lld rows x %d components exceed the 32-bit row index", what, (long long)(ry * rz), f->ncomp);
    return AXS_OK;
}

static int same_shape(const axs_fab *a, const axs_fab *b, const char *what)
{
    AXS_REQUIRE(a->dtype == b->dtype && a->nx == b->nx && a->ny == b->ny && a->nz == b->nz, AXS_ERR_INVALID_ARGUMENT,
                "%s: boxes differ in dtype or valid extent", what);
    return AXS_OK;
}

int level_fill_ghosts(void *data, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g, int ncomp,
                      cudaStream_t st)
{
    const int64_t n = (int64_t)(nx + 16) * (ny + 4) * nz * ncomp;
    if (dtype == AXS_F64)
        level_fill_ghosts_kernel<double><<<grid_for(n), 256, 0, st>>>(static_cast<double *>(data), nx, ny, nz, g, ncomp);
    else
        level_fill_ghosts_kernel<float><<<grid_for(n), 256, 0, st>>>(static_cast<float *>(data), nx, ny, nz, g, ncomp);
    return launch_status("level_fill_ghosts");
}

// Between a level and a contiguous (4, nz, ny, nx) device array (to_level: the
// array into the level, padding included; else the level's valid cells out).
int level_copy_contiguous(void *lv, void *arr, int32_t dtype, int nx, int ny, int nz, const LevelGeom &g,
                          int to_level, cudaStream_t st)
{
    const int sms = device_sm_count() > 0 ? device_sm_count() : 148;
    const int64_t rows = to_level ? (int64_t)(ny + 4) * nz * 4 : (int64_t)ny * nz * 4;
    const int grid = (int)std::min<int64_t>(rows, (int64_t)sms * 16);
    const int threads = nx + 16 <= 128 ? 128 : 256;
    if (dtype == AXS_F64) {
        if (to_level)
            level_scatter_kernel<double><<<grid, threads, 0, st>>>(static_cast<double *>(lv),
                                                                   static_cast<const double *>(arr), nx, ny, nz, g);
        else
            level_gather_kernel<double><<<grid, threads, 0, st>>>(static_cast<const double *>(lv),
                                                                  static_cast<double *>(arr), nx, ny, nz, g);
    } else {
        if (to_level)
            level_scatter_kernel<float><<<grid, threads, 0, st>>>(static_cast<float *>(lv),
                                                                  static_cast<const float *>(arr), nx, ny, nz, g);
        else
            level_gather_kernel<float><<<grid, threads, 0, st>>>(static_cast<const float *>(lv),
                                                                 static_cast<float *>(arr), nx, ny, nz, g);
    }
    return launch_status(to_level ? "level scatter" : "level gather");
}

int level_copy_fab(void *lv, int32_t dtype, const LevelGeom &g, const axs_fab &f, int to_level, cudaStream_t st)
{
    const int64_t n = (int64_t)f.nx * f.ny * f.nz * 4;
    if (dtype == AXS_F64)
        level_from_fab_kernel<double><<<grid_for(n), 256, 0, st>>>(static_cast<double *>(lv), g, f, to_level);
    else
        level_from_fab_kernel<float><<<grid_for(n), 256, 0, st>>>(static_cast<float *>(lv), g, f, to_level);
    return launch_status("level_copy_fab");
}

}  // namespace axs

using namespace axs;

extern "C" {

int axs_level_handoff_rescale(const axs_level *lv, double R_pre, double R_pre_prime, double R_main,
                              double R_main_prime, void *stream)
{
    AXS_REQUIRE(lv != nullptr && lv->state != nullptr, AXS_ERR_INVALID_ARGUMENT, "null level");
    AXS_REQUIRE(R_pre != 0.0, AXS_ERR_INVALID_ARGUMENT, "R_pre must be nonzero");
    LevelGeom g;
    int rc = level_geom(lv->dtype, lv->nx, lv->ny, lv->nz, g);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t n = (int64_t)lv->nx * lv->ny * lv->nz;
    // the reference holds R and R' as amrex::Real
    if (lv->dtype == AXS_F64)
        level_handoff_kernel<double><<<grid_for(n), 256, 0, st>>>(static_cast<double *>(lv->state), lv->nx, lv->ny,
                                                                  lv->nz, g, R_pre, R_pre_prime, R_main, R_main_prime);
    else
        level_handoff_kernel<float><<<grid_for(n), 256, 0, st>>>(static_cast<float *>(lv->state), lv->nx, lv->ny,
                                                                 lv->nz, g, (float)R_pre, (float)R_pre_prime,
                                                                 (float)R_main, (float)R_main_prime);
    if ((rc = launch_status("handoff rescale"))) return rc;
    return level_fill_ghosts(lv->state, lv->dtype, lv->nx, lv->ny, lv->nz, g, 4, st);
}

static int count_nonfinite(const void *base, int32_t dtype, int nx, int ny, int nz, int64_t js, int64_t ks,
                           int64_t cs, int64_t *count_dev, cudaStream_t st)
{
    AXS_REQUIRE(count_dev != nullptr, AXS_ERR_INVALID_ARGUMENT, "null count");
    AXS_CUDA_CHECK(cudaMemsetAsync(count_dev, 0, sizeof(int64_t), st));
    const int64_t n = (int64_t)nx * ny * nz;
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(count_dev);
    if (dtype == AXS_F64)
        count_nonfinite_kernel<double><<<grid_for(n), 256, 0, st>>>(static_cast<const double *>(base), nx, ny, nz, js,
                                                                    ks, cs, cnt);
    else
        count_nonfinite_kernel<float><<<grid_for(n), 256, 0, st>>>(static_cast<const float *>(base), nx, ny, nz, js,
                                                                   ks, cs, cnt);
    return launch_status("non-finite count");
}

int axs_count_nonfinite(const axs_fab *state, int64_t *count_dev, void *stream)
{
    int rc = validate_fab(state, "state", 4, 0);
    if (rc) return rc;
    const size_t es = dtype_size(state->dtype);
    const char *base = static_cast<const char *>(state->data) +
                       (state->ng + state->ng * state->jstride + state->ng * state->kstride) * es;
    return count_nonfinite(base, state->dtype, state->nx, state->ny, state->nz, state->jstride, state->kstride,
                           state->cstride, count_dev, (cudaStream_t)stream);
}

int axs_level_count_nonfinite(const axs_level *lv, int64_t *count_dev, void *stream)
{
    AXS_REQUIRE(lv != nullptr && lv->state != nullptr, AXS_ERR_INVALID_ARGUMENT, "null level");
    LevelGeom g;
    int rc = level_geom(lv->dtype, lv->nx, lv->ny, lv->nz, g);
    if (rc) return rc;
    const char *base = static_cast<const char *>(lv->state) + (g.ox + g.oy * g.js) * dtype_size(lv->dtype);
    return count_nonfinite(base, lv->dtype, lv->nx, lv->ny, lv->nz, g.js, g.ks, g.cs, count_dev,
                           (cudaStream_t)stream);
}

int axs_eval_rhs(const axs_fab *soln, const axs_fab *rhs, double dx, const axs_rhs_coeffs *c, void *stream)
{
    int rc = validate_fab(soln, "soln", 4, 2);
    if (rc) return rc;
    if ((rc = validate_fab(rhs, "rhs", 4, 0))) return rc;
    if ((rc = same_shape(soln, rhs, "eval_rhs"))) return rc;
    AXS_REQUIRE(c != nullptr, AXS_ERR_INVALID_ARGUMENT, "null coefficients");
    AXS_REQUIRE(dx > 0.0, AXS_ERR_INVALID_ARGUMENT, "dx must be positive");
    if ((rc = rows_fit(soln, "eval_rhs"))) return rc;
    const int g = grid_rows((int64_t)soln->ny * soln->nz);
    const double one_over_dx2 = 1.0 / (dx * dx);
    cudaStream_t st = (cudaStream_t)stream;
    if (soln->dtype == AXS_F64)
        eval_rhs_f64_kernel<<<g, 256, 0, st>>>(*soln, *rhs, one_over_dx2, c->kappa, c->lambda, c->R2);
    else {
        const dim3 grid((soln->nx + 31) / 32, (soln->ny + 7) / 8, (soln->nz + 63) / 64), block(32, 8);
        const bool w16 = soln->ng % 4 == 2 && soln->jstride % 4 == 0 && soln->kstride % 4 == 0 &&
                         soln->cstride % 4 == 0 && (uintptr_t)soln->data % 16 == 0 && soln->nx % 32 == 0 &&
                         soln->ny % 8 == 0;
        const float k = (float)c->kappa, l = (float)c->lambda, r2 = (float)c->R2;
        if (w16)
            eval_rhs_f32_zmarch_kernel<8, 64, 2, true><<<grid, block, 0, st>>>(*soln, *rhs, (float)one_over_dx2, k, l,
                                                                               r2);
        else
            eval_rhs_f32_zmarch_kernel<8, 64, 2, false><<<grid, block, 0, st>>>(*soln, *rhs, (float)one_over_dx2, k, l,
                                                                                r2);
    }
    return launch_status("eval_rhs");
}

static int fill_ghosts(const axs_fab *f, int with_z, cudaStream_t st)
{
    int rc = rows_fit(f, "periodic fill");
    if (rc) return rc;
    AXS_REQUIRE(f->ncomp <= 65535, AXS_ERR_UNSUPPORTED, "periodic fill: more than 65535 components");
    const int64_t gy = f->ny + 2 * f->ng, rows = (with_z ? 2 * f->ng * gy : 0) + (int64_t)f->nz * 2 * f->ng;
    const int64_t cells = (int64_t)f->ny * f->nz * 2 * f->ng;
    const int64_t gr = grid_rows(rows), gc = grid_for(cells);
    const dim3 grid((unsigned)(gr > gc ? gr : gc), (unsigned)f->ncomp);
    if (f->dtype == AXS_F64)
        fill_periodic_kernel<double><<<grid, 256, 0, st>>>(*f, with_z);
    else
        fill_periodic_kernel<float><<<grid, 256, 0, st>>>(*f, with_z);
    return launch_status(with_z ? "fill_periodic_ghosts" : "fill_periodic_ghosts_xy");
}

int axs_fill_periodic_ghosts_xy(const axs_fab *f, void *stream)
{
    int rc = validate_fab(f, "fab", 1, 0);
    if (rc) return rc;
    if (f->ng == 0) return AXS_OK;
    AXS_REQUIRE(f->ng <= f->nx && f->ng <= f->ny, AXS_ERR_UNSUPPORTED, "periodic fill needs ng <= box extent");
    return fill_ghosts(f, 0, (cudaStream_t)stream);
    return launch_status("fill_periodic_ghosts_xy");
}

static int copy_z_planes(const axs_fab *f, int32_t z0, int32_t nplanes, void *buf, int to_buf, cudaStream_t st)
{
    int rc = validate_fab(f, "fab", 1, 0);
    if (rc) return rc;
    AXS_REQUIRE(buf != nullptr, AXS_ERR_INVALID_ARGUMENT, "null plane buffer");
    AXS_REQUIRE(nplanes > 0 && z0 >= -f->ng && z0 + nplanes <= f->nz + f->ng, AXS_ERR_INVALID_ARGUMENT,
                "planes %d .. %d outside the FAB's z range %d .. %d", z0, z0 + nplanes - 1, -f->ng,
                f->nz + f->ng - 1);
    if ((rc = rows_fit(f, "z plane copy"))) return rc;
    const int g = grid_rows((int64_t)(f->ny + 2 * f->ng) * nplanes * f->ncomp);
    if (f->dtype == AXS_F64)
        copy_z_planes_kernel<double><<<g, 256, 0, st>>>(*f, z0, nplanes, static_cast<double *>(buf), to_buf);
    else
        copy_z_planes_kernel<float><<<g, 256, 0, st>>>(*f, z0, nplanes, static_cast<float *>(buf), to_buf);
    return launch_status("z plane copy");
}

int axs_fab_pack_z_planes(const axs_fab *f, int32_t z0, int32_t nplanes, void *buf, void *stream)
{
    return copy_z_planes(f, z0, nplanes, buf, 1, (cudaStream_t)stream);
}

int axs_fab_unpack_z_planes(const axs_fab *f, int32_t z0, int32_t nplanes, const void *buf, void *stream)
{
    return copy_z_planes(f, z0, nplanes, const_cast<void *>(buf), 0, (cudaStream_t)stream);
}

int axs_fill_periodic_ghosts(const axs_fab *f, void *stream)
{
    int rc = validate_fab(f, "fab", 1, 0);
    if (rc) return rc;
    if (f->ng == 0) return AXS_OK;
    AXS_REQUIRE(f->ng <= f->nx && f->ng <= f->ny && f->ng <= f->nz, AXS_ERR_UNSUPPORTED,
                "periodic fill needs ng <= box extent");
    return fill_ghosts(f, 1, (cudaStream_t)stream);
}

int axs_lincomb(const axs_fab *dst, const axs_fab *x, double b, const axs_fab *y, void *stream)
{
    int rc;
    if ((rc = validate_fab(dst, "dst", 1, 0)) || (rc = validate_fab(x, "x", 1, 0)) || (rc = validate_fab(y, "y", 1, 0)))
        return rc;
    if ((rc = same_shape(dst, x, "lincomb")) || (rc = same_shape(dst, y, "lincomb"))) return rc;
    const int nc = dst->ncomp < x->ncomp ? (dst->ncomp < y->ncomp ? dst->ncomp : y->ncomp)
                                         : (x->ncomp < y->ncomp ? x->ncomp : y->ncomp);
    if ((rc = rows_fit(dst, "lincomb"))) return rc;
    const int g = grid_rows((int64_t)dst->ny * dst->nz * nc);
    cudaStream_t st = (cudaStream_t)stream;
    if (dst->dtype == AXS_F64)
        lincomb_kernel<double><<<g, 256, 0, st>>>(*dst, *x, b, *y, nc);
    else
        lincomb_kernel<float><<<g, 256, 0, st>>>(*dst, *x, (float)b, *y, nc);
    return launch_status("lincomb");
}

int axs_rk4_combine(const axs_fab *dst, const axs_fab *uold, const axs_fab *k1, const axs_fab *k2, const axs_fab *k3,
                    const axs_fab *k4, double dt, void *stream)
{
    const axs_fab *all[6] = {dst, uold, k1, k2, k3, k4};
    const char *names[6] = {"dst", "uold", "k1", "k2", "k3", "k4"};
    for (int q = 0; q < 6; ++q) {
        int rc = validate_fab(all[q], names[q], 4, 0);
        if (rc) return rc;
        if (q && (rc = same_shape(dst, all[q], "rk4_combine"))) return rc;
    }
    int rc = rows_fit(dst, "rk4_combine");
    if (rc) return rc;
    const int g = grid_rows((int64_t)dst->ny * dst->nz * 4);
    cudaStream_t st = (cudaStream_t)stream;
    if (dst->dtype == AXS_F64)
        rk4_combine_kernel<double><<<g, 256, 0, st>>>(*dst, *uold, *k1, *k2, *k3, *k4, dt / 6.0, 4);
    else
        rk4_combine_kernel<float><<<g, 256, 0, st>>>(*dst, *uold, *k1, *k2, *k3, *k4, (float)(dt / 6.0), 4);
    return launch_status("rk4_combine");
}

}  // extern "C"
