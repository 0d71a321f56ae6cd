// Per-site operations of the two fused RK4 sweeps (see rk4_level.cu for the
// two-sweep factorisation of classic RK4) and their host-side constants,
// shared by the single-level and the ensemble advance.
#pragma once

#include "sweep.cuh"

namespace axs {

// Stage arithmetic of sweep A on V sites: from the Laplacians and centre
// values of (psi1, psi2, Pi1, Pi2) to the increments
//   o = (d3_1, d3_2, d4_1, d4_2, E_1, E_2, Q_1, Q_2),
//   d3 = h/2 Pi + h^2/4 F1            (S3 = psi + d3)
//   d4 = h Pi + h^2/2 F2              (S4 = psi + d4)
//   E  = h Pi + h^2/6 (F1 + F2 + L)   (psi_{n+1} = psi + E + h^2/6 (F3 - L))
//   Q  = h/6 F1 + h/3 F2 + h/2 L      (Pi_{n+1}  = Pi + Q + h/3 (F3 - L) + h/6 (F4 - L))
// with L = lap psi_n. Every stored quantity is an increment, of the size of
// h Pi rather than of psi: sweep B rebuilds S3, S4 and the new state by adding
// them to psi_n, Pi_n, so the state is rounded once per step at its own scale
// and the stage Laplacians lap S = L + lap d never see a stage value rounded
// at the scale of psi. The separate sweeps and the fused steps all call this
// function, so their results agree bit for bit.
//
// COMP, the compensated FP32 step: every product with a step fraction c
// (h, h/2, h^2/4, ...) is formed as (c + c_lo) x = fma(c_lo, x, fma(c, x, y)),
// c_lo the FP32 remainder of c. FP32 rounds each fraction once for the whole
// run, in the same direction at every site, a bias of ~3e-8 per step that the
// plain form integrates (with the Laplacian weights' remainders, lap_pair).
template <typename T, int V, bool COMP = false>
__device__ __forceinline__ void stage_a(const SweepArgs<T> &a, const T (&lap)[4][V], const T (&ctr)[4][V],
                                        T (&o)[8][V])
{
    if constexpr (kPackedPairs<T, V>) {
        // the expressions below, two sites per instruction
#pragma unroll
        for (int v = 0; v < V; v += 2) {
            const F2 p1(ctr[0][v], ctr[0][v + 1]), p2(ctr[1][v], ctr[1][v + 1]);
            const F2 q1(ctr[2][v], ctr[2][v + 1]), q2(ctr[3][v], ctr[3][v + 1]);
            const F2 l0(lap[0][v], lap[0][v + 1]), l1(lap[1][v], lap[1][v + 1]);
            const F2 l2(lap[2][v], lap[2][v + 1]), l3(lap[3][v], lap[3][v + 1]);
            const F2 hh(a.h_half);
            F2 f11, f12, f21, f22;
            F2 r[8];
            rhs_pair(a.c1, p1, p2, l0, l1, f11, f12);
            if constexpr (!COMP) {
                const F2 c1 = fma(hh, q1, p1), c2 = fma(hh, q2, p2);
                rhs_pair(a.c2, c1, c2, fma(hh, l2, l0), fma(hh, l3, l1), f21, f22);
                const F2 hq1 = F2(a.h) * q1, hq2 = F2(a.h) * q2;
                r[0] = fma(F2(a.h2_quarter), f11, hh * q1);
                r[1] = fma(F2(a.h2_quarter), f12, hh * q2);
                r[2] = fma(F2(a.h2_half), f21, hq1);
                r[3] = fma(F2(a.h2_half), f22, hq2);
                r[4] = fma(F2(a.h2_sixth), (f11 + f21) + l0, hq1);
                r[5] = fma(F2(a.h2_sixth), (f12 + f22) + l1, hq2);
                r[6] = fma(hh, l0, fma(F2(a.h_third), f21, F2(a.h_sixth) * f11));
                r[7] = fma(hh, l1, fma(F2(a.h_third), f22, F2(a.h_sixth) * f12));
            } else {
                auto cm = [](F2 c, F2 cl, F2 x, F2 y) { return fma(cl, x, fma(c, x, y)); };  // (c + c_lo) x + y
                const F2 hhl(a.h_half_lo), z(0.f, 0.f);
                const F2 c1 = cm(hh, hhl, q1, p1), c2 = cm(hh, hhl, q2, p2);
                rhs_pair(a.c2, c1, c2, cm(hh, hhl, l2, l0), cm(hh, hhl, l3, l1), f21, f22);
                const F2 hq1 = cm(F2(a.h), F2(a.h_lo), q1, z), hq2 = cm(F2(a.h), F2(a.h_lo), q2, z);
                const F2 hhq1 = cm(hh, hhl, q1, z), hhq2 = cm(hh, hhl, q2, z);
                const F2 H2Q(a.h2_quarter), H2Ql(a.h2_quarter_lo), H2H(a.h2_half), H2Hl(a.h2_half_lo);
                const F2 H26(a.h2_sixth), H26l(a.h2_sixth_lo), H3(a.h_third), H3l(a.h_third_lo);
                const F2 H6(a.h_sixth), H6l(a.h_sixth_lo);
                r[0] = cm(H2Q, H2Ql, f11, hhq1);
                r[1] = cm(H2Q, H2Ql, f12, hhq2);
                r[2] = cm(H2H, H2Hl, f21, hq1);
                r[3] = cm(H2H, H2Hl, f22, hq2);
                r[4] = cm(H26, H26l, (f11 + f21) + l0, hq1);
                r[5] = cm(H26, H26l, (f12 + f22) + l1, hq2);
                r[6] = cm(hh, hhl, l0, cm(H3, H3l, f21, cm(H6, H6l, f11, z)));
                r[7] = cm(hh, hhl, l1, cm(H3, H3l, f22, cm(H6, H6l, f12, z)));
            }
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                o[c][v] = r[c].v.x;
                o[c][v + 1] = r[c].v.y;
            }
        }
    } else {
        static_assert(!COMP, "the compensated step is built for packed FP32 pairs");
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const T p1 = ctr[0][v], p2 = ctr[1][v], q1 = ctr[2][v], q2 = ctr[3][v];
            T f11, f12, f21, f22;
            rhs_pair(a.c1, p1, p2, lap[0][v], lap[1][v], f11, f12);  // F1 = F(t, psi_n)
            // F2 = F(t + h/2, chi), chi = psi_n + h/2 Pi_n, lap(chi) = lap(psi) + h/2 lap(Pi)
            const T c1 = fma(a.h_half, q1, p1), c2 = fma(a.h_half, q2, p2);
            rhs_pair(a.c2, c1, c2, fma(a.h_half, lap[2][v], lap[0][v]), fma(a.h_half, lap[3][v], lap[1][v]), f21, f22);
            const T hq1 = a.h * q1, hq2 = a.h * q2;
            o[0][v] = fma(a.h2_quarter, f11, a.h_half * q1);                      // d3
            o[1][v] = fma(a.h2_quarter, f12, a.h_half * q2);
            o[2][v] = fma(a.h2_half, f21, hq1);                                   // d4
            o[3][v] = fma(a.h2_half, f22, hq2);
            o[4][v] = fma(a.h2_sixth, (f11 + f21) + lap[0][v], hq1);              // E
            o[5][v] = fma(a.h2_sixth, (f12 + f22) + lap[1][v], hq2);
            o[6][v] = fma(a.h_half, lap[0][v], fma(a.h_third, f21, a.h_sixth * f11));  // Q
            o[7][v] = fma(a.h_half, lap[1][v], fma(a.h_third, f22, a.h_sixth * f12));
        }
    }
}

// Stage arithmetic of sweep B on V sites: from the Laplacians and centre
// values of (d3_1, d3_2, d4_1, d4_2) and the pointwise
// pq = (E_1, E_2, Q_1, Q_2, psi1, psi2, Pi1, Pi2) of the step's start to
// o = (psi1, psi2, Pi1, Pi2) at its end. With S = psi_n + d, the stage RHS is
// F(S) = L + G with G = lap d + (kappa - lambda/2 (|S|^2 - R^2)) S; the L
// parts are already in E and Q.
template <typename T, int V, typename PQ, bool COMP = false>
__device__ __forceinline__ void stage_b(const SweepArgs<T> &a, const T (&lap)[4][V], const T (&ctr)[4][V],
                                        const PQ &pq, T (&o)[4][V])
{
    if constexpr (kPackedPairs<T, V>) {
        // the expressions below, two sites per instruction
#pragma unroll
        for (int v = 0; v < V; v += 2) {
            auto pr = [&](const T (&x)[V]) { return F2(x[v], x[v + 1]); };
            const F2 p1 = pr(pq[4]), p2 = pr(pq[5]);
            F2 g31, g32, g41, g42;
            rhs_pair(a.c2, p1 + pr(ctr[0]), p2 + pr(ctr[1]), pr(lap[0]), pr(lap[1]), g31, g32);
            rhs_pair(a.c4, p1 + pr(ctr[2]), p2 + pr(ctr[3]), pr(lap[2]), pr(lap[3]), g41, g42);
            F2 r[4];
            if constexpr (!COMP) {
                r[0] = p1 + fma(F2(a.h2_sixth), g31, pr(pq[0]));
                r[1] = p2 + fma(F2(a.h2_sixth), g32, pr(pq[1]));
                r[2] = pr(pq[6]) + fma(F2(a.h_sixth), g41, fma(F2(a.h_third), g31, pr(pq[2])));
                r[3] = pr(pq[7]) + fma(F2(a.h_sixth), g42, fma(F2(a.h_third), g32, pr(pq[3])));
            } else {
                auto cm = [](F2 c, F2 cl, F2 x, F2 y) { return fma(cl, x, fma(c, x, y)); };
                const F2 H26(a.h2_sixth), H26l(a.h2_sixth_lo), H3(a.h_third), H3l(a.h_third_lo);
                const F2 H6(a.h_sixth), H6l(a.h_sixth_lo);
                r[0] = p1 + cm(H26, H26l, g31, pr(pq[0]));
                r[1] = p2 + cm(H26, H26l, g32, pr(pq[1]));
                r[2] = pr(pq[6]) + cm(H6, H6l, g41, cm(H3, H3l, g31, pr(pq[2])));
                r[3] = pr(pq[7]) + cm(H6, H6l, g42, cm(H3, H3l, g32, pr(pq[3])));
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                o[c][v] = r[c].v.x;
                o[c][v + 1] = r[c].v.y;
            }
        }
    } else {
        static_assert(!COMP, "the compensated step is built for packed FP32 pairs");
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const T p1 = pq[4][v], p2 = pq[5][v];
            T g31, g32, g41, g42;
            rhs_pair(a.c2, p1 + ctr[0][v], p2 + ctr[1][v], lap[0][v], lap[1][v], g31, g32);  // F3 - L at S3
            rhs_pair(a.c4, p1 + ctr[2][v], p2 + ctr[3][v], lap[2][v], lap[3][v], g41, g42);  // F4 - L at S4
            o[0][v] = p1 + fma(a.h2_sixth, g31, pq[0][v]);
            o[1][v] = p2 + fma(a.h2_sixth, g32, pq[1][v]);
            o[2][v] = pq[6][v] + fma(a.h_sixth, g41, fma(a.h_third, g31, pq[2][v]));
            o[3][v] = pq[7][v] + fma(a.h_sixth, g42, fma(a.h_third, g32, pq[3][v]));
        }
    }
}

// Sweep A: stencil on (psi_n, Pi_n); writes d3, d4 (with periodic copies) and E, Q.
template <bool COMP> struct ForwardAT {
    static constexpr int kPointwise = 0;
    static constexpr bool kLambdaGrad = false;
    static constexpr bool kComp = COMP;
    template <typename T, int V, bool HINT, typename PQ>
    __device__ static void apply(const SweepArgs<T> &a, const BoxGeom &b, const T (&lap)[4][V],
                                 const T (&ctr)[4][V], const PQ &, int64_t off, int x, int y, LamAcc<T> &,
                                 uint64_t pol)
    {
        T o[8][V];
        stage_a<T, V, COMP>(a, lap, ctr, o);
#pragma unroll
        for (int c = 0; c < 4; ++c)
            store_with_copies<T, V, HINT>(a.out[c], off, x, y, b.nx, b.ny, b.js, o[c], pol, b.periodic);
#pragma unroll
        for (int c = 4; c < 8; ++c) st_out<T, V, HINT>(a.out[c] + off, o[c], pol);
    }
};

// Sweep B: stencil on (d3, d4), pointwise (E, Q) and (psi_n, Pi_n); writes
// psi_{n+1}, Pi_{n+1} (over psi_n, Pi_n: each site reads its own inputs first).
template <bool COMP> struct ForwardBT {
    static constexpr int kPointwise = 8;
    static constexpr bool kLambdaGrad = false;
    static constexpr bool kComp = COMP;
    template <typename T, int V, bool HINT, typename PQ>
    __device__ static void apply(const SweepArgs<T> &a, const BoxGeom &b, const T (&lap)[4][V],
                                 const T (&ctr)[4][V], const PQ &pq, int64_t off, int x, int y, LamAcc<T> &,
                                 uint64_t pol)
    {
        T o[4][V];
        stage_b<T, V, PQ, COMP>(a, lap, ctr, pq, o);
#pragma unroll
        for (int c = 0; c < 4; ++c)
            store_with_copies<T, V, HINT>(a.out[c], off, x, y, b.nx, b.ny, b.js, o[c], pol, b.periodic);
    }
};
using ForwardA = ForwardAT<false>;
using ForwardB = ForwardBT<false>;

// Host: step constants shared by every box (Laplacian weights for dx, RK4 step
// fractions) and the bounded-wait limit of this launch.
template <typename T> inline void fill_step_constants(SweepArgs<T> &a, double dx, double dt)
{
    const double inv_dx2 = 1.0 / (dx * dx);
    a.wA = T((4.0 / 3.0) * inv_dx2);
    a.wB = T((-1.0 / 12.0) * inv_dx2);
    a.wC = T(-7.5 * inv_dx2);
    a.h = T(dt);
    a.h_half = T(0.5 * dt);
    a.h2_quarter = T(0.25 * dt * dt);
    a.h2_half = T(0.5 * dt * dt);
    a.h_sixth = T(dt / 6.0);
    a.h_third = T(dt / 3.0);
    a.h2_sixth = T(dt * dt / 6.0);
    a.wA_lo = T((4.0 / 3.0) * inv_dx2 - (double)a.wA);
    a.wB_lo = T((-1.0 / 12.0) * inv_dx2 - (double)a.wB);
    a.h_lo = T(dt - (double)a.h);
    a.h_half_lo = T(0.5 * dt - (double)a.h_half);
    a.h2_quarter_lo = T(0.25 * dt * dt - (double)a.h2_quarter);
    a.h2_half_lo = T(0.5 * dt * dt - (double)a.h2_half);
    a.h_sixth_lo = T(dt / 6.0 - (double)a.h_sixth);
    a.h_third_lo = T(dt / 3.0 - (double)a.h_third);
    a.h2_sixth_lo = T(dt * dt / 6.0 - (double)a.h2_sixth);
    a.wait_polls = device_wait_polls();
}

// Host: kappa, lambda/2 and R^2 at one stage time (the reference's
// specific_eval_rhs coefficients, AxionStringsLevel.cpp:850-921).
template <typename T> inline StageCoef<T> stage_coef(const axs_background &bg, double tau)
{
    axs_rhs_coeffs c;
    rhs_coeffs(bg, tau, c);
    return StageCoef<T>{T(c.kappa), T(0.5 * c.lambda), T(c.R2)};
}

}  // namespace axs
