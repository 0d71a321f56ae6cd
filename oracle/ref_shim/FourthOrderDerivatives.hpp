// Stand-in for GRTeclyn's FourthOrderDerivatives (third-party, absent from
// the reference tree) -- test infrastructure. Restates the published
// centred fourth-order 5-point weights: diff2 (1/12, 4/3, 5/2) * 1/dx^2,
// diff1 (1/12, 2/3) * 1/dx, evaluated in double; d1_scalar returns the three
// directional diff1 of one component, indexable as grad(dir).
#pragma once
#include "axs_amrex_shim.H"

#define FOR(IDX) for (int IDX = 0; IDX < AMREX_SPACEDIM; ++IDX)

class FourthOrderDerivatives
{
  public:
    const double m_dx;

  private:
    const double m_one_over_dx;
    const double m_one_over_dx2;

  public:
    explicit FourthOrderDerivatives(double dx)
        : m_dx(dx), m_one_over_dx(1.0 / dx), m_one_over_dx2(1.0 / (dx * dx))
    {
    }

    amrex::Real diff2(const amrex::Real *in, amrex::Long s) const
    {
        const double wf = 8.33333333333333333333e-2;
        const double wn = 1.33333333333333333333e+0;
        const double wl = 2.50000000000000000000e+0;
        return amrex::Real((-wf * double(in[-2 * s]) + wn * double(in[-s]) - wl * double(in[0]) +
                            wn * double(in[s]) - wf * double(in[2 * s])) *
                           m_one_over_dx2);
    }

    amrex::Real diff1(const amrex::Real *in, amrex::Long s) const
    {
        const double wf = 8.33333333333333333333e-2;
        const double wn = 6.66666666666666666667e-1;
        return amrex::Real((wf * double(in[-2 * s]) - wn * double(in[-s]) + wn * double(in[s]) -
                            wf * double(in[2 * s])) *
                           m_one_over_dx);
    }

    template <class A>
    amrex::Array1D<amrex::Real, 0, 2> d1_scalar(int i, int j, int k, const A &a, int comp) const
    {
        const amrex::Real *p = a.ptr(i, j, k) + comp * a.stride.a[2];
        return amrex::Array1D<amrex::Real, 0, 2>{{diff1(p, 1), diff1(p, a.stride.a[0]), diff1(p, a.stride.a[1])}};
    }
};
