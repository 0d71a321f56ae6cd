// Plaquette winding arithmetic shared by the string finder (diagnostics.cu)
// and the refinement tagger (tagging.cu): the reference's double arithmetic
// (PlaquetteWinding.hpp:24-51) and a single-precision fast path whose fold
// decisions are provably the same away from a 1e-5 band around +-pi.
#pragma once

#include "axs_internal.cuh"

namespace axs {

// wrap_angle_diff (PlaquetteWinding.hpp:24-38): fold into (-pi, pi]; flags
// edges within 1e-12 of +-pi, where a different atan2 could round the other way.
__device__ __forceinline__ double wrap_diff(double d, int &near_tie)
{
    const double pi = 3.14159265358979323846;
    const double two_pi = 2.0 * pi;
    if (fabs(fabs(d) - pi) < 1e-12) near_tie = 1;
    d = fmod(d, two_pi);
    if (d <= -pi)
        d = __dadd_rn(d, two_pi);
    else if (d > pi)
        d = __dsub_rn(d, two_pi);
    return d;
}

// PlaquetteWinding.hpp:42-51 literally, on double phases.
__device__ __forceinline__ int winding4(double t1, double t2, double t3, double t4, int &ties)
{
    int n1 = 0, n2 = 0, n3 = 0, n4 = 0;
    const double a = wrap_diff(__dsub_rn(t2, t1), n1);
    const double b = wrap_diff(__dsub_rn(t3, t2), n2);
    const double c = wrap_diff(__dsub_rn(t4, t3), n3);
    const double d = wrap_diff(__dsub_rn(t1, t4), n4);
    ties += n1 + n2 + n3 + n4;
    const double total = __dadd_rn(__dadd_rn(__dadd_rn(a, b), c), d);
    return (int)llround(__ddiv_rn(total, 2.0 * 3.14159265358979323846));
}

// Winding from single-precision phases. With every edge difference at least
// 1e-5 away from +-pi the fold decisions of the reference's double arithmetic
// are forced (the phases here are within ~1e-6 of the double ones), and the
// winding is #(d <= -pi) - #(d > pi). Returns false when an edge is inside
// that band: the caller then redoes the plaquette in double.
__device__ __forceinline__ bool winding4_fast(float t1, float t2, float t3, float t4, int &w)
{
    const float pi = 3.14159265f, band = 1e-5f;
    const float d[4] = {t2 - t1, t3 - t2, t4 - t3, t1 - t4};
    int up = 0, down = 0;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const float a = fabsf(d[e]);
        if (fabsf(a - pi) < band) return false;
        up += d[e] < -pi;
        down += d[e] > pi;
    }
    w = up - down;
    return true;
}


// The three windings at the low corner of a cell from its 7 corner phases
// (StringFinder.hpp:45-68 order: xy, yz, zx), float fast path first; false
// when the caller must redo the cell in double.
__device__ __forceinline__ bool cell_windings_fast(float f000, float f100, float f110, float f010, float f001,
                                                   float f101, float f011, int (&w)[3])
{
    return winding4_fast(f000, f100, f110, f010, w[0]) && winding4_fast(f000, f010, f011, f001, w[1]) &&
           winding4_fast(f000, f001, f101, f100, w[2]);
}

__device__ __forceinline__ void cell_windings_double(double d000, double d100, double d110, double d010, double d001,
                                                     double d101, double d011, int (&w)[3], int &ties)
{
    w[0] = winding4(d000, d100, d110, d010, ties);
    w[1] = winding4(d000, d010, d011, d001, ties);
    w[2] = winding4(d000, d001, d101, d100, ties);
}

}  // namespace axs
