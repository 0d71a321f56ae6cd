// Minimal single-box stand-in for the parts of AMReX that the reference's
// hot-path headers use -- TEST INFRASTRUCTURE ONLY.
//
// Written for this project so that the reference's own, unchanged headers
// (AxionStringsRHS.impl.hpp, StringFinder.hpp, EnergyKernel.hpp,
// VelocityKernel.hpp, FourierIC.hpp) compile on the host and can be run on
// small periodic boxes to produce golden vectors. Only what those headers
// touch is provided: Array4/Array1D views, a one-box MultiFab/iMultiFab,
// ReduceOps/ReduceData as a sequential (k, j, i) loop, no-op
// ParallelDescriptor reductions, and a naive-DFT FFT::R2C whose backward
// transform follows the FFTW c2r convention (complex inverse over the
// non-contiguous axes, then a real inverse along x that keeps only the real
// part of the kx = 0 and kx = nx/2 terms).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#ifndef AXS_REF_REAL
#define AXS_REF_REAL double
#endif

#define AMREX_GPU_DEVICE
#define AMREX_GPU_HOST_DEVICE
#define AMREX_FORCE_INLINE inline
#define AMREX_SPACEDIM 3
#define AMREX_D_DECL(a, b, c) a, b, c
#define BL_PROFILE(x)

namespace amrex
{
using Real = AXS_REF_REAL;
using Long = long;
template <class T> using Vector = std::vector<T>;

template <class T> constexpr const T &max(const T &a, const T &b) { return a < b ? b : a; }
template <class T> constexpr const T &min(const T &a, const T &b) { return b < a ? b : a; }

struct Dim3
{
    int x, y, z;
};

template <class T, int XLO, int XHI> struct Array1D
{
    T arr[XHI - XLO + 1];
    T &operator()(int i) { return arr[i - XLO]; }
    const T &operator()(int i) const { return arr[i - XLO]; }
};

struct Array4Stride
{
    Long a[3];
};

template <class T> struct CellData
{
    T *p;
    Long nstride;
    T &operator[](int n) const { return p[n * nstride]; }
};

// View of one FAB: (i,j,k) in [begin, end), component-major, x fastest.
template <class T> struct Array4
{
    T *p{nullptr};
    Array4Stride stride{{0, 0, 0}}; // {jstride, kstride, nstride}
    Dim3 begin{0, 0, 0};
    Dim3 end{0, 0, 0};
    int ncomp{0};

    Array4() = default;
    Array4(T *ap, Dim3 b, Dim3 e, int nc) : p(ap), begin(b), end(e), ncomp(nc)
    {
        stride.a[0] = Long(e.x - b.x);
        stride.a[1] = stride.a[0] * Long(e.y - b.y);
        stride.a[2] = stride.a[1] * Long(e.z - b.z);
    }
    template <class U>
    Array4(const Array4<U> &o) : p(o.p), stride(o.stride), begin(o.begin), end(o.end), ncomp(o.ncomp)
    {
    }
    Long offset(int i, int j, int k) const
    {
        return Long(i - begin.x) + Long(j - begin.y) * stride.a[0] + Long(k - begin.z) * stride.a[1];
    }
    T *ptr(int i, int j, int k) const { return p + offset(i, j, k); }
    T &operator()(int i, int j, int k, int n = 0) const { return p[offset(i, j, k) + n * stride.a[2]]; }
    CellData<T> cellData(int i, int j, int k) const { return CellData<T>{ptr(i, j, k), stride.a[2]}; }
};

// TagBox: only the tag type and values a tagging functor writes.
struct TagBox
{
    using TagType = char;
    static constexpr TagType CLEAR = 0, BUF = 1, SET = 2;
};

template <class T> struct MultiArray4
{
    Array4<T> a;
    const Array4<T> &operator[](int) const { return a; }
};

struct IntVect
{
    int v[3];
    explicit IntVect(int s = 0) : v{s, s, s} {}
    IntVect(int a, int b, int c) : v{a, b, c} {}
    int operator[](int d) const { return v[d]; }
};

struct Box
{
    int n[3];
    int length(int d) const { return n[d]; }
    Long numPts() const { return Long(n[0]) * n[1] * n[2]; }
    IntVect smallEnd() const { return IntVect(0); }
    IntVect bigEnd() const { return IntVect(n[0] - 1, n[1] - 1, n[2] - 1); }
};
struct BoxArray
{
    Box box;
};
struct DistributionMapping
{
};
struct Periodicity
{
};

struct Geometry
{
    Box dom;
    const Box &Domain() const { return dom; }
};

// One periodic box of nx*ny*nz valid cells, `ng` ghosts per side.
template <class T> struct FabArrayShim
{
    std::vector<T> owned;
    T *data{nullptr};
    int n[3]{0, 0, 0};
    int ng{0};
    int nc{0};

    FabArrayShim() = default;
    FabArrayShim(T *d, int nx, int ny, int nz, int a_ng, int a_nc) : data(d), n{nx, ny, nz}, ng(a_ng), nc(a_nc) {}
    FabArrayShim(const BoxArray &ba, const DistributionMapping &, int a_nc, int a_ng)
        : n{ba.box.n[0], ba.box.n[1], ba.box.n[2]}, ng(a_ng), nc(a_nc)
    {
        owned.assign(size_t(n[0] + 2 * ng) * (n[1] + 2 * ng) * (n[2] + 2 * ng) * nc, T{});
        data = owned.data();
    }
    Array4<T> array() const
    {
        return Array4<T>(data, Dim3{-ng, -ng, -ng}, Dim3{n[0] + ng, n[1] + ng, n[2] + ng}, nc);
    }
    MultiArray4<T const> const_arrays() const { return MultiArray4<T const>{Array4<T const>(array())}; }
    MultiArray4<T> arrays() const { return MultiArray4<T>{array()}; }
    template <class I> Array4<T const> const_array(const I &) const { return Array4<T const>(array()); }
    BoxArray boxArray() const { return BoxArray{Box{{n[0], n[1], n[2]}}}; }
    DistributionMapping DistributionMap() const { return {}; }
    void setVal(T v)
    {
        auto a = array();
        for (int c = 0; c < nc; ++c)
            for (int k = -ng; k < n[2] + ng; ++k)
                for (int j = -ng; j < n[1] + ng; ++j)
                    for (int i = -ng; i < n[0] + ng; ++i) a(i, j, k, c) = v;
    }
    void mult(T s, int comp, int ncomp)
    {
        auto a = array();
        for (int c = comp; c < comp + ncomp; ++c)
            for (int k = 0; k < n[2]; ++k)
                for (int j = 0; j < n[1]; ++j)
                    for (int i = 0; i < n[0]; ++i) a(i, j, k, c) *= s;
    }
    static T Dot(const FabArrayShim &x, int xc, const FabArrayShim &y, int yc, int ncomp, int)
    {
        double s = 0.0;
        auto ax = x.array();
        auto ay = y.array();
        for (int c = 0; c < ncomp; ++c)
            for (int k = 0; k < x.n[2]; ++k)
                for (int j = 0; j < x.n[1]; ++j)
                    for (int i = 0; i < x.n[0]; ++i) s += double(ax(i, j, k, xc + c)) * double(ay(i, j, k, yc + c));
        return T(s);
    }
};
using MultiFab = FabArrayShim<Real>;
using iMultiFab = FabArrayShim<int>;

// ParallelFor over the valid cells of a one-box FabArray (box number 0), in (k, j, i) order.
template <class FA, class F> void ParallelFor(const FA &fa, F &&f)
{
    for (int k = 0; k < fa.n[2]; ++k)
        for (int j = 0; j < fa.n[1]; ++j)
            for (int i = 0; i < fa.n[0]; ++i) f(0, i, j, k);
}

namespace Gpu
{
inline void streamSynchronize() {}
} // namespace Gpu

// The single box of a one-box FabArray.
struct MFIter
{
    Box box;
    bool valid{true};
    template <class FA> explicit MFIter(const FA &fa) : box{{fa.n[0], fa.n[1], fa.n[2]}} {}
    bool isValid() const { return valid; }
    MFIter &operator++()
    {
        valid = false;
        return *this;
    }
    const Box &validbox() const { return box; }
};

struct ReduceOpSum
{
};

template <class... Ts> struct ReduceData
{
    using Type = std::tuple<Ts...>;
    Type acc{};
    template <class Ops> explicit ReduceData(Ops &) {}
    template <class Ops> Type value(Ops &) const { return acc; }
    template <std::size_t... I> void add(const Type &t, std::index_sequence<I...>)
    {
        ((std::get<I>(acc) += std::get<I>(t)), ...);
    }
    void add(const Type &t) { add(t, std::index_sequence_for<Ts...>{}); }
};

template <class... Ops> struct ReduceOps
{
    // Sequential reduction over the valid cells in (k, j, i) order.
    template <class MF, class RD, class F> void eval(const MF &mf, IntVect, RD &rd, F &&f)
    {
        for (int k = 0; k < mf.n[2]; ++k)
            for (int j = 0; j < mf.n[1]; ++j)
                for (int i = 0; i < mf.n[0]; ++i) rd.add(f(0, i, j, k));
    }
};

template <std::size_t N, class... Ts> auto get(const std::tuple<Ts...> &t) { return std::get<N>(t); }

namespace ParallelDescriptor
{
inline void ReduceLongSum(long &) {}
inline void ReduceLongSum(long *, int) {}
inline void ReduceRealSum(double &) {}
inline void ReduceRealSum(double *, int) {}
inline void ReduceRealSum(float &) {}
inline void ReduceRealSum(float *, int) {}
} // namespace ParallelDescriptor

template <class T> struct GpuComplex
{
    T re{0}, im{0};
    GpuComplex() = default;
    GpuComplex(T r, T i) : re(r), im(i) {}
    T real() const { return re; }
    T imag() const { return im; }
};

namespace FFT
{
// Naive-DFT stand-in for amrex::FFT::R2C (small boxes only).
template <class T> struct R2C
{
    Box dom;
    using cMF = FabArrayShim<GpuComplex<T>>;
    explicit R2C(const Box &d) : dom(d) {}
    std::pair<BoxArray, DistributionMapping> getSpectralDataLayout() const
    {
        return {BoxArray{Box{{dom.n[0] / 2 + 1, dom.n[1], dom.n[2]}}}, DistributionMapping{}};
    }
    // Unnormalised forward transform, X_k = sum_x f(x) exp(-2 pi i k.x/N), kx >= 0 stored.
    void forward(const FabArrayShim<T> &in, cMF &out)
    {
        const int nx = dom.n[0], ny = dom.n[1], nz = dom.n[2], nxh = nx / 2 + 1;
        const double two_pi = 2.0 * 3.14159265358979323846;
        auto a = in.array();
        // x transform per (y, z) row, then (y, z) per kx
        std::vector<std::complex<double>> row(size_t(nxh) * ny * nz);
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int i = 0; i < nxh; ++i)
                {
                    std::complex<double> s = 0.0;
                    for (int x = 0; x < nx; ++x)
                    {
                        const double ph = -two_pi * double(i) * x / nx;
                        s += double(a(x, y, z, 0)) * std::complex<double>(std::cos(ph), std::sin(ph));
                    }
                    row[i + size_t(nxh) * (y + size_t(ny) * z)] = s;
                }
        auto o = out.array();
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nxh; ++i)
                {
                    std::complex<double> s = 0.0;
                    for (int z = 0; z < nz; ++z)
                        for (int y = 0; y < ny; ++y)
                        {
                            const double ph = -two_pi * (double(j) * y / ny + double(k) * z / nz);
                            s += row[i + size_t(nxh) * (y + size_t(ny) * z)] *
                                 std::complex<double>(std::cos(ph), std::sin(ph));
                        }
                    o(i, j, k, 0) = GpuComplex<T>(T(s.real()), T(s.imag()));
                }
    }
    template <class F> void forwardThenBackward(const MultiFab &, MultiFab &out, F fill)
    {
        const int nx = dom.n[0], ny = dom.n[1], nz = dom.n[2], nxh = nx / 2 + 1;
        std::vector<std::complex<double>> spec(size_t(nxh) * ny * nz);
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nxh; ++i)
                {
                    GpuComplex<T> c;
                    fill(i, j, k, c);
                    spec[i + size_t(nxh) * (j + size_t(ny) * k)] = {double(c.re), double(c.im)};
                }
        const double two_pi = 2.0 * 3.14159265358979323846;
        // complex inverse over (ky, kz) for each kx
        std::vector<std::complex<double>> mid(size_t(nxh) * ny * nz);
        for (int i = 0; i < nxh; ++i)
            for (int y = 0; y < ny; ++y)
                for (int z = 0; z < nz; ++z)
                {
                    std::complex<double> s = 0.0;
                    for (int k = 0; k < nz; ++k)
                        for (int j = 0; j < ny; ++j)
                        {
                            const double ph = two_pi * (double(j) * y / ny + double(k) * z / nz);
                            s += spec[i + size_t(nxh) * (j + size_t(ny) * k)] * std::complex<double>(std::cos(ph), std::sin(ph));
                        }
                    mid[i + size_t(nxh) * (y + size_t(ny) * z)] = s;
                }
        auto a = out.array();
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x)
                {
                    double s = 0.0;
                    for (int i = 0; i < nxh; ++i)
                    {
                        const std::complex<double> m = mid[i + size_t(nxh) * (y + size_t(ny) * z)];
                        const double ph = two_pi * double(i) * x / nx;
                        const double re = m.real() * std::cos(ph) - m.imag() * std::sin(ph);
                        const bool self_conj = (i == 0) || (2 * i == nx);
                        s += self_conj ? (i == 0 ? m.real() : m.real() * std::cos(ph)) : 2.0 * re;
                    }
                    a(x, y, z, 0) = T(s);
                }
    }
};
} // namespace FFT
} // namespace amrex
