// level_demo -- a C++ host program driving the GB300 hot path through the C
// ABI with axs_host::AxionStringsLevel: read an initial state, advance it with
// the fused RK4, write the final state and print the post-timestep
// diagnostics as one JSON line.
//
//   axs_level_demo <f32|f64> nx ny nz dx a_inv c0 lambda0 tau_i dt nsteps ic.bin out.bin
//
// ic.bin: float64 (4, nz, ny, nx) psi1, psi2, Pi1, Pi2; out.bin: the final
// state (4, nz, ny, nx) in the run's precision.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#include "axs_level.hpp"

int main(int argc, char **argv)
{
    if (argc != 14) {
        std::fprintf(stderr, "usage: %s f32|f64 nx ny nz dx a_inv c0 lambda0 tau_i dt nsteps ic.bin out.bin\n",
                     argv[0]);
        return 2;
    }
    const bool f64 = std::string(argv[1]) == "f64";
    const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]);
    const double dx = std::atof(argv[5]), a_inv = std::atof(argv[6]), c0 = std::atof(argv[7]);
    const double lambda0 = std::atof(argv[8]), tau_i = std::atof(argv[9]), dt = std::atof(argv[10]);
    const int nsteps = std::atoi(argv[11]);
    const size_t n = (size_t)4 * nx * ny * nz;
    std::vector<double> ic(n);
    {
        std::ifstream f(argv[12], std::ios::binary);
        if (!f.read(reinterpret_cast<char *>(ic.data()), (std::streamsize)(n * sizeof(double)))) {
            std::fprintf(stderr, "cannot read %s\n", argv[12]);
            return 2;
        }
    }
    try {
        axs_background bg{};
        bg.kind = AXS_BG_EXPANDING;
        bg.a_inv = a_inv;
        bg.c0 = c0;
        bg.lambda_scale = lambda0;
        axs_host::AxionStringsLevel level(nx, ny, nz, dx, bg, tau_i, f64 ? AXS_F64 : AXS_F32);
        std::vector<char> host(n * (f64 ? 8 : 4));
        if (f64) {
            std::memcpy(host.data(), ic.data(), n * 8);
        } else {
            float *h = reinterpret_cast<float *>(host.data());
            for (size_t i = 0; i < n; ++i) h[i] = (float)ic[i];
        }
        level.set_state(host.data());
        level.advance(dt, nsteps);
        const axs_host::Diagnostics d = level.specific_post_timestep();
        level.get_state(host.data());
        std::ofstream o(argv[13], std::ios::binary);
        o.write(host.data(), (std::streamsize)host.size());
        std::printf("{\"tau\": %.17g, \"n_p_plain\": %lld, \"n_p_weighted\": %lld, \"xi_plain\": %.17g, "
                    "\"rho_tot_unscreened\": %.17g, \"rho_tot_screened\": %.17g, \"vel_count\": %lld, "
                    "\"mean_gamma_sq_v_sq\": %.17g, \"energy_sums\": [",
                    level.tau(), (long long)d.n_p_plain, (long long)d.n_p_weighted, d.xi_plain, d.rho_tot_unscreened,
                    d.rho_tot_screened, (long long)d.vel_count, d.mean_gamma_sq_v_sq);
        for (int i = 0; i < 14; ++i) std::printf("%s%.17g", i ? ", " : "", d.energy_sums[i]);
        std::printf("]}\n");
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
