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
template <typename T, int V>
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
            rhs_pair(a.c1, p1, p2, l0, l1, f11, f12);
            const F2 c1 = fma(hh, q1, p1), c2 = fma(hh, q2, p2);
            rhs_pair(a.c2, c1, c2, fma(hh, l2, l0), fma(hh, l3, l1), f21, f22);
            const F2 hq1 = F2(a.h) * q1, hq2 = F2(a.h) * q2;
            const F2 r[8] = {fma(F2(a.h2_quarter), f11, hh * q1),
                             fma(F2(a.h2_quarter), f12, hh * q2),
                             fma(F2(a.h2_half), f21, hq1),
                             fma(F2(a.h2_half), f22, hq2),
                             fma(F2(a.h2_sixth), (f11 + f21) + l0, hq1),
                             fma(F2(a.h2_sixth), (f12 + f22) + l1, hq2),
                             fma(hh, l0, fma(F2(a.h_third), f21, F2(a.h_sixth) * f11)),
                             fma(hh, l1, fma(F2(a.h_third), f22, F2(a.h_sixth) * f12))};
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                o[c][v] = r[c].v.x;
                o[c][v + 1] = r[c].v.y;
            }
        }
    } else {
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
template <typename T, int V, typename PQ>
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
            const F2 r[4] = {p1 + fma(F2(a.h2_sixth), g31, pr(pq[0])),
                             p2 + fma(F2(a.h2_sixth), g32, pr(pq[1])),
                             pr(pq[6]) + fma(F2(a.h_sixth), g41, fma(F2(a.h_third), g31, pr(pq[2]))),
                             pr(pq[7]) + fma(F2(a.h_sixth), g42, fma(F2(a.h_third), g32, pr(pq[3])))};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                o[c][v] = r[c].v.x;
                o[c][v + 1] = r[c].v.y;
            }
        }
    } else {
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
struct ForwardA {
    static constexpr int kPointwise = 0;
    static constexpr bool kLambdaGrad = false;
    template <typename T, int V, bool HINT, typename PQ>
    __device__ static void apply(const SweepArgs<T> &a, const BoxGeom &b, const T (&lap)[4][V],
                                 const T (&ctr)[4][V], const PQ &, int64_t off, int x, int y, double &,
                                 uint64_t pol)
    {
        T o[8][V];
        stage_a<T, V>(a, lap, ctr, o);
#pragma unroll
        for (int c = 0; c < 4; ++c)
            store_with_copies<T, V, HINT>(a.out[c], off, x, y, b.nx, b.ny, b.js, o[c], pol, b.periodic);
#pragma unroll
        for (int c = 4; c < 8; ++c) st_out<T, V, HINT>(a.out[c] + off, o[c], pol);
    }
};

// Sweep B: stencil on (d3, d4), pointwise (E, Q) and (psi_n, Pi_n); writes
// psi_{n+1}, Pi_{n+1} (over psi_n, Pi_n: each site reads its own inputs first).
struct ForwardB {
    static constexpr int kPointwise = 8;
    static constexpr bool kLambdaGrad = false;
    template <typename T, int V, bool HINT, typename PQ>
    __device__ static void apply(const SweepArgs<T> &a, const BoxGeom &b, const T (&lap)[4][V],
                                 const T (&ctr)[4][V], const PQ &pq, int64_t off, int x, int y, double &,
                                 uint64_t pol)
    {
        T o[4][V];
        stage_b<T, V>(a, lap, ctr, pq, o);
#pragma unroll
        for (int c = 0; c < 4; ++c)
            store_with_copies<T, V, HINT>(a.out[c], off, x, y, b.nx, b.ny, b.js, o[c], pol, b.periodic);
    }
};

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
