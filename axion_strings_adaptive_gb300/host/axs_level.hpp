// axs_level.hpp -- C++ host side of the GB300 hot path: the reference level's
// hooks (AxionStrings/AxionStringsLevel.hpp:18-46) over the C ABI of axs.h.
//
// A C++ application (the AMReX/GRTeclyn code, or any driver) keeps its own
// control flow and calls:
//   specific_eval_rhs       -> axs_eval_rhs         (AxionStringsLevel.cpp:850-921)
//   advance                 -> axs_level_rk4_advance (GRTeclyn's RK4 level step, fused)
//   specific_post_timestep  -> axs_level_diagnostics (AxionStringsLevel.cpp:1256-1434:
//                              N_p, xi, the 14 energy sums, <gamma^2 v^2>)
// Device memory is owned by this class (cudaMalloc at construction, nothing
// allocated per call); every library status is turned into an exception, the
// C++ counterpart of the reference's amrex::Abort.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>

#include "axs.h"

namespace axs_host {

inline void check(int status)
{
    if (status != AXS_OK) throw std::runtime_error(std::string("axs: ") + axs_last_error());
}

inline void cuda_check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

class DeviceBuffer {
public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes) : bytes_(bytes)
    {
        if (bytes) cuda_check(cudaMalloc(&p_, bytes), "cudaMalloc");
    }
    DeviceBuffer(DeviceBuffer &&o) noexcept : p_(std::exchange(o.p_, nullptr)), bytes_(o.bytes_) {}
    DeviceBuffer &operator=(DeviceBuffer &&o) noexcept
    {
        std::swap(p_, o.p_);
        std::swap(bytes_, o.bytes_);
        return *this;
    }
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    ~DeviceBuffer()
    {
        if (p_) cudaFree(p_);
    }
    void *get() const { return p_; }
    size_t bytes() const { return bytes_; }

private:
    void *p_ = nullptr;
    size_t bytes_ = 0;
};

// specific_post_timestep's single-level quantities.
struct Diagnostics {
    int64_t n_p_plain = 0, n_p_weighted = 0;
    double xi_plain = 0, xi_weighted = 0;
    double energy_sums[14] = {};
    double rho_tot_unscreened = 0, rho_tot_screened = 0;
    double mean_gamma_sq_v_sq = 0;
    int64_t vel_count = 0;
    int64_t n_near_tie = 0;
};

class AxionStringsLevel {
public:
    // One periodic box of nx*ny*nz cells of spacing dx; conformal time
    // tau = tau_i + time (AxionStringsLevel.hpp:65-72).
    AxionStringsLevel(int nx, int ny, int nz, double dx, const axs_background &bg, double tau_i, int32_t dtype,
                      cudaStream_t stream = nullptr)
        : bg_(bg), tau_i_(tau_i), stream_(stream)
    {
        check(axs_level_layout_for(dtype, nx, ny, nz, &layout_));
        es_ = dtype == AXS_F64 ? 8 : 4;
        state_ = DeviceBuffer((size_t)layout_.state_bytes);
        work_ = DeviceBuffer((size_t)layout_.work_bytes);
        cuda_check(cudaMemset(work_.get(), 0, work_.bytes()), "cudaMemset");
        lv_ = axs_level{state_.get(), work_.get(), dtype, nx, ny, nz, dx, 0, 0};
        staging_ = DeviceBuffer((size_t)4 * nx * ny * nz * es_);
        int64_t sb = 0;
        check(axs_diagnostics_scratch_bytes(nx, ny, nz, &sb));
        scratch_ = DeviceBuffer((size_t)sb);
        result_ = DeviceBuffer(sizeof(axs_diag_result));
    }

    double tau() const { return tau_i_ + time_; }
    double time() const { return time_; }
    const axs_level &level() const { return lv_; }
    void set_tile_config(int32_t id) { lv_.tile_config = id; }
    // the compensated FP32 step (AXS_LEVEL_COMPENSATED_FP32; no effect in FP64)
    void set_compensated(bool on)
    {
        lv_.flags = on ? (lv_.flags | AXS_LEVEL_COMPENSATED_FP32) : (lv_.flags & ~AXS_LEVEL_COMPENSATED_FP32);
    }

    // Valid cells (4, nz, ny, nx) of the level's dtype from / to host memory.
    void set_state(const void *host)
    {
        cuda_check(cudaMemcpy(staging_.get(), host, staging_.bytes(), cudaMemcpyHostToDevice), "cudaMemcpy");
        const axs_fab f = dense_fab();
        check(axs_level_import_fab(&lv_, &f, stream_));
        cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    }

    void get_state(void *host) const
    {
        const axs_fab f = dense_fab();
        check(axs_level_export_fab(&lv_, &f, stream_));
        cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        cuda_check(cudaMemcpy(host, staging_.get(), staging_.bytes(), cudaMemcpyDeviceToHost), "cudaMemcpy");
    }

    // AxionStringsLevel::specific_eval_rhs on caller FABs (AMReX Array4 layout).
    void specific_eval_rhs(const axs_fab &soln, const axs_fab &rhs, double a_time) const
    {
        axs_rhs_coeffs c;
        check(axs_background_rhs_coeffs(&bg_, tau_i_ + a_time, &c));
        check(axs_eval_rhs(&soln, &rhs, lv_.dx, &c, stream_));
    }

    // nsteps classic-RK4 steps of the level (fused sweeps), asynchronous.
    void advance(double dt, int nsteps)
    {
        check(axs_level_rk4_advance(&lv_, &bg_, tau_i_, time_, dt, nsteps, stream_));
        time_ += nsteps * dt;
    }

    // The diagnostics of specific_post_timestep at the current time (synchronises).
    Diagnostics specific_post_timestep(int32_t masking_scheme = AXS_MASK_A, double threshold = 0.8,
                                       bool per_cell_fp32 = false)
    {
        check(axs_level_device_status(&lv_, stream_));
        axs_background_values v;
        check(axs_background_eval(&bg_, tau(), &v));
        const double rpr = bg_.kind == AXS_BG_FLAT ? 0.0 : v.R_prime_over_R;
        axs_diag_params p{lv_.dx, v.R, v.lambda, rpr, v.m_r, masking_scheme, threshold, AXS_BOUNDARY_PERIODIC,
                          1, 1, 1, per_cell_fp32 ? 1 : 0};
        check(axs_level_diagnostics(&lv_, &p, nullptr, static_cast<axs_diag_result *>(result_.get()), nullptr, 0,
                                    scratch_.get(), (int64_t)scratch_.bytes(), stream_));
        axs_diag_result r;
        cuda_check(cudaMemcpyAsync(&r, result_.get(), sizeof(r), cudaMemcpyDeviceToHost, stream_), "cudaMemcpy");
        cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        Diagnostics d;
        const double n_cells = (double)lv_.nx * lv_.ny * lv_.nz, L_tilde = lv_.nx * lv_.dx;
        d.n_p_plain = r.n_p_plain;
        d.n_p_weighted = r.n_p_weighted;
        d.xi_plain = axs_xi_from_plaquette_count((double)r.n_p_plain, lv_.dx, L_tilde, bg_.a_inv, tau());
        d.xi_weighted = axs_xi_from_plaquette_count((double)r.n_p_weighted, lv_.dx, L_tilde, bg_.a_inv, tau());
        std::memcpy(d.energy_sums, r.energy_sums, sizeof(d.energy_sums));
        d.rho_tot_unscreened = r.energy_sums[0] / n_cells;  // EnergyKernel.hpp:239-268
        d.rho_tot_screened = r.energy_sums[12] > 0.0 ? r.energy_sums[1] / r.energy_sums[12] : 0.0;
        d.vel_count = r.vel_count;
        d.mean_gamma_sq_v_sq = r.vel_count > 0 ? r.vel_sum / (double)r.vel_count : 0.0;
        d.n_near_tie = r.n_near_tie;
        return d;
    }

private:
    axs_fab dense_fab() const
    {
        const int64_t nx = lv_.nx, ny = lv_.ny, nz = lv_.nz;
        return axs_fab{staging_.get(), lv_.dtype, lv_.nx, lv_.ny, lv_.nz, 0, 4, nx, nx * ny, nx * ny * nz};
    }

    axs_background bg_;
    double tau_i_, time_ = 0.0;
    cudaStream_t stream_;
    axs_level_layout layout_{};
    size_t es_ = 4;
    DeviceBuffer state_, work_, staging_, scratch_, result_;
    axs_level lv_{};
};

}  // namespace axs_host
