/*
 * axs.h -- C ABI of the GB300-native axion-string hot path.
 *
 * One shared library (libaxs_gb300.so, sm_103a) replaces the per-level hot
 * path of the AMReX/GRTeclyn axion-string code:
 *   (a) the complex-scalar RHS and its classic-RK4 time step,
 *   (b) the plaquette-winding string finder (counts + compacted pierced list),
 *   (c) the energy, string-velocity and xi reductions.
 *
 * Conventions
 *   - Every entry point returns an axs_status (0 = AXS_OK). No C++ exception
 *     crosses the ABI. axs_last_error() gives a message for the calling thread.
 *   - The caller owns every buffer. Device pointers are plain CUDA device
 *     addresses; `stream` is a cudaStream_t (NULL = legacy default stream).
 *   - Device entry points are asynchronous on `stream` and never synchronise,
 *     allocate or free, so they can be captured in a CUDA graph. Results that
 *     the reference returned by value (plaquette counts, energy sums) are
 *     written to caller-provided DEVICE memory.
 *   - Arguments are validated on the host before anything is launched; a
 *     failed validation launches nothing.
 *   - One CUDA device per process: kernels' shared-memory limits and
 *     occupancy figures are set up on the first call that launches them and
 *     assumed for every later call. Make that first call outside stream
 *     capture.
 *
 * Each declaration names the reference interface it replaces (paths relative
 * to the reference project root).
 */
#ifndef AXS_H
#define AXS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AXS_ABI_VERSION 2

typedef enum axs_status {
    AXS_OK = 0,
    AXS_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, bad enum */
    AXS_ERR_UNSUPPORTED = 2,      /* shape / layout the kernels do not handle */
    AXS_ERR_ALIGNMENT = 3,        /* pointer or stride not 16-byte aligned */
    AXS_ERR_WORKSPACE = 4,        /* caller-provided scratch too small */
    AXS_ERR_CUDA = 5,             /* a CUDA runtime/driver call failed */
    AXS_ERR_DEVICE_TIMEOUT = 6,   /* a bounded device-side wait gave up */
    AXS_ERR_CAPACITY = 7          /* pierced list truncated (counts stay exact) */
} axs_status;

typedef enum axs_dtype { AXS_F32 = 1, AXS_F64 = 2 } axs_dtype;

/* Component order of the state (AxionStrings/StateVariables.hpp:9-17). */
enum { AXS_C_PSI1 = 0, AXS_C_PSI2 = 1, AXS_C_PI1 = 2, AXS_C_PI2 = 3, AXS_NUM_VARS = 4 };

/* One AMReX FArrayBox viewed through plain pointers: cell (i,j,k) of
 * component c, i in [-ng, nx+ng) etc., lives at
 *   data + (i+ng) + (j+ng)*jstride + (k+ng)*kstride + c*cstride   (elements).
 * This is exactly amrex::Array4's layout (AxionStringsRHS.impl.hpp:29-36),
 * so a box of a MultiFab maps with zero copies. */
typedef struct axs_fab {
    void *data;
    int32_t dtype; /* axs_dtype */
    int32_t nx, ny, nz, ng;
    int32_t ncomp;
    int64_t jstride, kstride, cstride;
} axs_fab;

/* RHS coefficients resolved on the host at one stage time
 * (AxionStringsLevel.cpp:856-907; AxionStringsRHS.hpp:32-36). */
typedef struct axs_rhs_coeffs {
    double kappa;  /* curvature_term_coeff(tau) */
    double lambda; /* lambda(tau) */
    double R2;     /* R(tau)^2 */
} axs_rhs_coeffs;

/* Background models behind the coefficients: Background.hpp:21-134 (power
 * law, c(tau) schedule with one switch), FlatBackground.hpp:26-44,
 * PreEvolutionBackground.hpp:37-78, plus the optional post-handoff
 * smoothstep blend of AxionStringsLevel.cpp:893-906. lambda_scale multiplies
 * lambda (the reference fixes lambda0 = 1, Background.hpp:37; 1.0 reproduces it). */
typedef enum axs_background_kind { AXS_BG_EXPANDING = 0, AXS_BG_FLAT = 1, AXS_BG_PRE_EVOLUTION = 2 } axs_background_kind;

typedef struct axs_background {
    int32_t kind; /* axs_background_kind */
    int32_t has_switch;
    double a_inv, c0, c1, tau_switch;
    double lambda_scale;
    double m_r;       /* flat: lambda = m_r^2 */
    double gamma_pre; /* pre-evolution: constant m_r/H */
    double blend_dtau, blend_tau_start, blend_lambda_start, blend_curv_start;
} axs_background;

typedef struct axs_background_values {
    double R, R_prime, kappa, lambda, H, R2, m_r, R_prime_over_R;
} axs_background_values;

/* ---------------------------------------------------------------------------
 * Host-side scalar models (no GPU needed)
 * ------------------------------------------------------------------------- */

/* Background::{R, R_prime, curvature_term_coeff, lambda, H} (Background.hpp:55-107)
 * and the coefficient resolution of specific_eval_rhs (AxionStringsLevel.cpp:856-907). */
int axs_background_eval(const axs_background *bg, double tau, axs_background_values *out);
int axs_background_rhs_coeffs(const axs_background *bg, double tau, axs_rhs_coeffs *out);
/* Background::tau_from_log_mr_over_h (Background.hpp:129-133). */
int axs_background_tau_from_log_mr_over_h(const axs_background *bg, double log_mr_over_h, double *tau);

/* XiFormula.hpp:33-59. */
double axs_xi_from_comoving_length(double ell_comoving, double L_tilde, double a_inv, double tau);
double axs_xi_from_plaquette_count(double N_p, double dx, double L_tilde, double a_inv, double tau);
double axs_plaquette_count_for_target_xi(double xi_target, int N, double L_tilde, double a_inv, double tau);

const char *axs_status_string(int status);
const char *axs_last_error(void);
int axs_abi_version(void);

/* Failure detection (no counterpart in the reference, whose CPU loops never
 * wait). Every device-side wait of the stencil kernels (a thread block waiting
 * for a TMA copy to land) gives up after a bounded number of polls; the kernel
 * then sets AXS_ERR_DEVICE_TIMEOUT in the status word that the *_device_status
 * calls report, waits (bounded again, with its own fixed limit) for its copies
 * still in flight and ends, so the CUDA context stays usable. The limit is
 * library-wide: AXS_DEFAULT_WAIT_POLLS until set here. 0 makes every such
 * wait give up at once, which lets a test drive the timeout path without
 * harming the device. Launches read the value when they are issued (a
 * captured graph keeps the value of its capture). The previous value goes to
 * *previous (nullable). */
#define AXS_DEFAULT_WAIT_POLLS 4194304u
int axs_set_device_wait_polls(uint32_t polls, uint32_t *previous);

/* ---------------------------------------------------------------------------
 * (a) RHS on AMReX FABs -- the drop-in for the level hook
 * ------------------------------------------------------------------------- */

/* Replaces the body of AxionStringsLevel::specific_eval_rhs
 * (AxionStringsLevel.cpp:909-920): AxionStringsRHS<FourthOrderDerivatives>
 * (AxionStringsRHS.impl.hpp:25-60) over the valid cells of one box.
 * `soln` needs ng >= 2 filled ghost layers; rhs may have any ng. */
int axs_eval_rhs(const axs_fab *soln, const axs_fab *rhs, double dx, const axs_rhs_coeffs *c,
                 void *stream);

/* Replaces MultiFab::FillBoundary(periodicity) for a single-box periodic
 * domain (AxionStringsLevel.cpp:820, :1255): fills every ghost cell. */
int axs_fill_periodic_ghosts(const axs_fab *f, void *stream);

/* The halo seam of a z-slab decomposition (one slab of a periodic box per GPU;
 * replaces the inter-rank part of FillBoundary, AxionStringsLevel.cpp:820,
 * :1255). Per RK stage a slab
 *   1. fills its x/y ghosts periodically (axs_fill_periodic_ghosts_xy, valid z
 *      planes only),
 *   2. packs its lowest and highest ng valid planes, x/y ghosts included
 *      (axs_fab_pack_z_planes with z0 = 0 and z0 = nz - ng),
 *   3. sends them to its lower / upper neighbour (NCCL or any transport of the
 *      caller's choice) and
 *   4. unpacks the planes it receives into its z ghosts (axs_fab_unpack_z_planes
 *      with z0 = -ng and z0 = nz),
 * after which axs_eval_rhs and axs_diagnostics (AXS_BOUNDARY_GHOSTS) run on the
 * slab as on the whole box. A buffer holds planes z0 .. z0 + nplanes - 1 of all
 * components, contiguous as (ncomp, nplanes, ny + 2 ng, nx + 2 ng). The
 * diagnostics' result holds the slab's raw sums (14 energy sums, the two
 * counts, the velocity sum and count): the all-reduce of those 18 scalars and an
 * exclusive prefix sum of n_listed for the pierced-list offsets give the whole
 * box (StringFinder.hpp:119-120, EnergyKernel.hpp:215, VelocityKernel.hpp:138-139). */
int axs_fill_periodic_ghosts_xy(const axs_fab *f, void *stream);
int axs_fab_pack_z_planes(const axs_fab *f, int32_t z0, int32_t nplanes, void *buf_dev, void *stream);
int axs_fab_unpack_z_planes(const axs_fab *f, int32_t z0, int32_t nplanes, const void *buf_dev, void *stream);

/* dst = x + b*y over the valid cells of all components: the stage combination
 * U_s = U_old + c_s dt k (AMReX MultiFab::LinComb in GRTeclyn's RK driver). */
int axs_lincomb(const axs_fab *dst, const axs_fab *x, double b, const axs_fab *y, void *stream);

/* Final classic-RK4 combination dst = uold + dt/6 (k1 + 2 k2 + 2 k3 + k4). */
int axs_rk4_combine(const axs_fab *dst, const axs_fab *uold, const axs_fab *k1, const axs_fab *k2,
                    const axs_fab *k3, const axs_fab *k4, double dt, void *stream);

/* ---------------------------------------------------------------------------
 * (a) Fused RK4 on a periodic level (TMA-staged two-sweep scheme)
 * ------------------------------------------------------------------------- */

/* Device layout of a periodic single-box level: component-major SoA planes,
 * x fastest, each xy plane padded in x and by 2 rows on either side in y, no
 * z padding. Element (x,y,z,c) sits at
 *   (x + x_offset) + (y + y_offset)*jstride + z*kstride + c*cstride.
 * x_offset puts x = 0 on a 128-byte boundary (32 floats / 16 doubles) and
 * jstride is a multiple of 128 bytes, so every row of valid cells starts a
 * cache line; the 8 columns left of x = 0 and right of x = nx-1 (the stencils
 * read 4; 8 fill whole 32-byte sectors) and the 2 rows outside y hold periodic
 * copies that the kernels keep current (padding corners excepted). `state` holds psi1, psi2, Pi1, Pi2; `work` holds 8
 * components of the same layout used between the two sweeps of a step, plus
 * a 256-byte status block. Both must be 128-byte aligned. */
typedef struct axs_level_layout {
    int64_t jstride, kstride, cstride; /* elements */
    int32_t x_offset, y_offset;       /* elements */
    int64_t state_bytes;              /* 4 components */
    int64_t work_bytes;               /* 8 components + status block */
} axs_level_layout;

typedef struct axs_level {
    void *state;
    void *work;
    int32_t dtype; /* axs_dtype */
    int32_t nx, ny, nz;
    double dx;
    int32_t tile_config; /* 0 = default sweep tiling for the dtype; 1..N = axs_level_tile_config_name(dtype, id) */
    int32_t flags;       /* AXS_LEVEL_* bits, 0 = none */
} axs_level;

/* axs_level.flags: FP32 steps with the FP32 remainders of the Laplacian weights
 * and the RK4 step fractions (h, h/2, h^2/4, ...) applied as second FMAs. FP32
 * rounds each of those constants once for the whole run and in the same
 * direction at every site; the plain step integrates that bias (at 512^3 over
 * 400 steps it is most of the FP32 run's departure from FP64 beyond FP32
 * storage rounding). The same state layout and entry points; about 7 % slower.
 * Ignored for FP64 levels. */
#define AXS_LEVEL_COMPENSATED_FP32 1

int axs_level_layout_for(int32_t dtype, int32_t nx, int32_t ny, int32_t nz, axs_level_layout *out);

/* Sweep tilings compiled into the library (vector width, tile, ring depth):
 * ids 1..axs_level_tile_config_count(dtype); id 0 names the default. An
 * autotuner can time each on the caller's level and set axs_level.tile_config. */
int axs_level_tile_config_count(int32_t dtype);
const char *axs_level_tile_config_name(int32_t dtype, int32_t id);

/* Periodic ghost columns/rows of the 4 state components (call after writing
 * the state's valid cells by any other means). */
int axs_level_fill_ghosts(const axs_level *lv, void *stream);

/* Copy between an AMReX FAB (any ng) and the level layout, valid cells only.
 * import also refreshes the level's ghosts. */
int axs_level_import_fab(const axs_level *lv, const axs_fab *src, void *stream);
int axs_level_export_fab(const axs_level *lv, const axs_fab *dst, void *stream);

/* The level's valid cells from / to a HOST array (4, nz, ny, nx) of its dtype
 * (pinned memory for asynchronous copies): one contiguous DMA copy each way,
 * staged in the level's work buffer, and one device pass between that staging
 * array and the level layout (upload also fills the periodic padding). The
 * work buffer holds stage values only inside a step, so do not call these
 * between axs_level_rk4_sweep(A) and (B) of one step, nor concurrently with a
 * step of the same level. For callers whose fields live in host memory. */
int axs_level_upload(const axs_level *lv, const void *host_state, void *stream);
int axs_level_download(const axs_level *lv, void *host_state, void *stream);

/* Replaces GRTeclyn's RK4 level advance (docs/conventions.md:239-245, driver
 * absent from the reference tree) together with nsteps x 4 calls of
 * specific_eval_rhs: advances the state by nsteps classic-RK4 steps of size
 * dt from t0, coefficients from `bg` at tau = tau_i + t_stage. Two sweeps
 * per step; async on `stream`. */
int axs_level_rk4_advance(const axs_level *lv, const axs_background *bg, double tau_i, double t0,
                          double dt, int32_t nsteps, void *stream);

/* One axs_level_rk4_advance step from time t written into dst_state (a buffer
 * of the level's state layout, axs_level_layout.state_bytes, 128-byte aligned,
 * overlapping neither the state nor the work buffer), padding included; the
 * level's state is left as it was. A subcycling driver that needs the coarse
 * state at both ends of a step keeps the two buffers and swaps them, instead of
 * copying the state before an in-place step. */
int axs_level_rk4_step_to(const axs_level *lv, void *dst_state, const axs_background *bg, double tau_i, double t,
                          double dt, void *stream);

/* One of the two sweeps of the step starting at time t (sweep 0 = A: reads the
 * state, writes the between-sweep components; sweep 1 = B: reads those, writes
 * the state). Sweep A then sweep B equals one axs_level_rk4_advance step; this
 * entry point lets a caller time or interleave the sweeps. */
int axs_level_rk4_sweep(const axs_level *lv, const axs_background *bg, double tau_i, double t, double dt,
                        int32_t sweep, void *stream);

/* Synchronises `stream` and reports (and clears) the level's device status
 * word: AXS_OK or AXS_ERR_DEVICE_TIMEOUT. */
int axs_level_device_status(const axs_level *lv, void *stream);

/* AxionStringsLevel::apply_pre_evolution_to_main_rescale (AxionStringsLevel.cpp:2027-2132):
 * in place on the level, in the field precision, kappa = R_main/R_pre,
 * psi <- kappa psi, Pi <- kappa^2 Pi + (psi/R_pre)(R_main' - kappa^2 R_pre'),
 * with R_pre, R_pre' at the end of pre-evolution and R_main, R_main' at tau_i.
 * The caller then shifts tau_i by -tau_pre_end and, optionally, sets the
 * axs_background blend fields (handoff transition). */
int axs_level_handoff_rescale(const axs_level *lv, double R_pre, double R_pre_prime, double R_main,
                              double R_main_prime, void *stream);

/* ---------------------------------------------------------------------------
 * Differentiation: discrete adjoint of the fused RK4 step (no counterpart in
 * the reference, which has no gradient code)
 * ------------------------------------------------------------------------- */

/* Bytes of the adjoint workspace for a level: 8 components of the level
 * layout (Fbar and the stage adjoints) plus per-block lambda0-gradient partials. */
int axs_level_adjoint_work_bytes(int32_t dtype, int32_t nx, int32_t ny, int32_t nz, int64_t *bytes);

/* Reverse one axs_level_rk4_advance step taken from time t: lv->state must
 * hold the state y_n at the start of that step (lv->work is overwritten with
 * its recomputed stage fields). `abar` (4 components, level layout, periodic
 * padding current) holds dL/dy_{n+1} on entry and dL/dy_n on return;
 * *lambda0_bar (device) is incremented by dL/dlambda0 through this step, where
 * lambda0 = bg->lambda_scale. Asynchronous on `stream`. */
int axs_level_rk4_adjoint_step(const axs_level *lv, void *abar, void *adj_work, int64_t adj_work_bytes,
                               const axs_background *bg, double tau_i, double t, double dt, double *lambda0_bar,
                               void *stream);

/* Smooth string-core loss of the level's state:
 *   L = sum_cells exp(-|psi/R|^2 / width) + mean_cells (theta'/R)^2,
 * theta' = (psi1 Pi2 - Pi1 psi2)/|psi|^2 -- the second term is the unscreened
 * axion kinetic energy density average (Energy.hpp:90-97). Writes L to
 * *loss_dev and, if `grad` is not NULL, dL/d(psi1, psi2, Pi1, Pi2) in the
 * level layout (padding filled). `scratch` needs 8 bytes x 4 x SMs. */
int axs_level_string_core_loss(const axs_level *lv, double R, double width, double *loss_dev, void *grad,
                               void *scratch, int64_t scratch_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * (b)+(c) Fused diagnostics pass
 * ------------------------------------------------------------------------- */

typedef enum axs_masking_scheme { AXS_MASK_NONE = 0, AXS_MASK_A = 1, AXS_MASK_B = 2 } axs_masking_scheme;
typedef enum axs_boundary { AXS_BOUNDARY_GHOSTS = 0, AXS_BOUNDARY_PERIODIC = 1 } axs_boundary;

typedef struct axs_diag_params {
    double dx;
    double R, lambda, R_prime_over_R, m_r; /* host-resolved at the snapshot tau */
    int32_t masking_scheme;                /* axs_masking_scheme (Masking.hpp:39-53) */
    double masking_threshold;
    int32_t boundary;                      /* axs_boundary */
    int32_t want_energy, want_plaquettes, want_velocity; /* want_plaquettes alone: the string
                                              finder (windings, counts, pierced list), its own
                                              lean kernel */
    int32_t per_cell_fp32;                 /* FP32 fields only: 0 = per-cell energy, masking and
                                              gamma^2 v^2 in double as the reference computes them
                                              (sums equal the reference's FLOAT build); 1 = per-cell
                                              terms in FP32, summed per work item in compensated
                                              FP32 and across items in FP64 (about 1e-8 relative;
                                              ~14x faster on GB300, whose FP64 rate is 1/64 of
                                              FP32). Windings and counts are exact either way. */
} axs_diag_params;

/* Written to device memory by the diagnostics pass. */
typedef struct axs_diag_result {
    double energy_sums[14]; /* EnergyKernel.hpp:196-199 order: rho, rho w, a_kin, a_kin w,
                               a_grad, a_grad w, r_kin, r_kin w, r_grad, r_grad w,
                               r_mass, r_mass w, w, n_cells */
    double vel_sum;         /* VelocityKernel.hpp: sum of gamma^2 v^2 at pierced corners */
    int64_t vel_count;      /* corners counted (4 per pierced plaquette) */
    int64_t n_p_plain;      /* StringFinder.hpp:76-122 */
    int64_t n_p_weighted;
    int64_t n_listed;       /* entries written to the pierced list (<= capacity) */
    int64_t n_near_tie;     /* plaquette edges with | |dtheta| - pi | < 1e-12: the
                               only edges where a different atan2 could round the
                               other way (bit-exactness caveat) */
    int64_t status;         /* AXS_OK or AXS_ERR_CAPACITY */
} axs_diag_result;

/* Scratch (device) bytes the diagnostics pass needs for a box of this size. */
int axs_diagnostics_scratch_bytes(int32_t nx, int32_t ny, int32_t nz, int64_t *bytes);

/* One pass over the valid cells computing, as requested:
 *   - count_plaquettes (StringFinder.hpp:76-122, windings of
 *     plaquette_windings_at :45-68 / PlaquetteWinding.hpp:42-51) and a
 *     compacted list of pierced plaquettes, entry = 4*(i + nx*(j + ny*k)) + plane
 *     (plane 0 = xy, 1 = yz, 2 = zx), order unspecified;
 *   - compute_total_energy_sums (EnergyKernel.hpp:106-233);
 *   - compute_velocity_at_pierced_corners (VelocityKernel.hpp:37-141).
 * `mask` (nullable, nx*ny*nz bytes, 1 = include) is the composite coverage mask.
 * Sums are accumulated in FP64, deterministically (fixed tree, no float atomics). */
int axs_diagnostics(const axs_fab *state, const axs_diag_params *p, const uint8_t *mask,
                    axs_diag_result *result_dev, int64_t *pierced_dev, int64_t pierced_capacity,
                    void *scratch_dev, int64_t scratch_bytes, void *stream);

/* Non-finite cells: how many valid cells have a component (psi1, psi2, Pi1,
 * Pi2) that is NaN or infinite, into *count_dev (a device int64, overwritten).
 * A run that has blown up (a step too long for the stencil, a bad initial
 * field) shows here before its diagnostics turn into NaN sums. The reference
 * has no such check (it aborts on bad parameters, AxionStringsLevel.cpp:349-352,
 * not on bad state). */
int axs_count_nonfinite(const axs_fab *state, int64_t *count_dev, void *stream);
int axs_level_count_nonfinite(const axs_level *lv, int64_t *count_dev, void *stream);

/* Same pass on a fused-RK4 level (periodic wrap in z, ghost copies in x/y). */
int axs_level_diagnostics(const axs_level *lv, const axs_diag_params *p, const uint8_t *mask,
                          axs_diag_result *result_dev, int64_t *pierced_dev,
                          int64_t pierced_capacity, void *scratch_dev, int64_t scratch_bytes,
                          void *stream);

/* axs_diagnostics for callers that cannot give this library device memory
 * (no counterpart in the reference, which has no GPU path): the per-block
 * partials live in a 256 KiB static device array inside the library instead of
 * caller scratch, and the call allocates nothing. A pass needs 256 bytes plus
 * 160 bytes per block, with at most 8 blocks per SM, so every box fits on
 * devices of up to 204 SMs (GB300 has 152); on larger devices boxes whose pass
 * would need more than the array are rejected with AXS_ERR_WORKSPACE. The
 * first call on each device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it for the life of the process; make that
 * first call before any stream capture on the device, and do not call it
 * again after a cudaDeviceReset of that device. All calls share the one array,
 * so calls whose work overlaps on the GPU (different streams or threads) race:
 * serialise them. */
int axs_diagnostics_static_scratch(const axs_fab *state, const axs_diag_params *p, const uint8_t *mask,
                                   axs_diag_result *result_dev, int64_t *pierced_dev, int64_t pierced_capacity,
                                   void *stream);

/* plaquette_winding (PlaquetteWinding.hpp:42-51) on n device quadruples
 * theta[4*q .. 4*q+3] -> w[q]: the device winding kernel on caller-chosen
 * phases (known-answer tests). */
int axs_plaquette_winding_batch(const double *theta_dev, int64_t n, int32_t *w_dev, void *stream);

/* ---------------------------------------------------------------------------
 * Refined patches (the scale path's fine level; the reference's AMR is AMReX /
 * GRTeclyn, absent from its tree): every patch refines one block^3 block of a
 * periodic coarse level by 2 (n = 2 block fine cells per side, spacing dx/2,
 * two fine steps per coarse step). Patches carry explicit ghost rings (6
 * columns in x, 4 rows / planes in y, z); their state / work arenas are laid
 * out like an ensemble's, padded position of valid (0,0,0) = (x_offset,
 * y_offset, z_offset) inside each patch box of patch_elems elements.
 * ------------------------------------------------------------------------- */
typedef struct axs_patch_layout {
    int64_t jstride, kstride, patch_elems, plane_elems;
    int32_t x_offset, y_offset, z_offset;
    int64_t state_bytes, work_bytes, table_bytes;
} axs_patch_layout;

typedef struct axs_patches {
    int32_t dtype;
    int32_t n;        /* fine cells per patch side */
    int32_t npatches;
    double dx;        /* fine spacing */
    void *state;      /* 4 component planes */
    void *work;       /* 8 component planes; may be NULL when axs_patches_layout reports
                         work_bytes = 0 (the fused step covers the patch size and count) */
    void *table;      /* written by axs_patches_init */
    int64_t state_bytes, work_bytes, table_bytes;
    int32_t capacity; /* patch slots each component plane is laid out for (>= npatches; 0 = npatches):
                         a regrid that changes npatches keeps every patch's data in place
                         (size the arenas with axs_patches_layout(dtype, n, capacity)) */
} axs_patches;

typedef struct axs_patch_plan {
    int64_t items_a, items_b;
    int32_t grid_a, grid_b;
} axs_patch_plan;

/* Device arrays tying patches to coarse blocks: patch_block[3 q .. 3 q + 2] =
 * block coordinates of patch q; block_patch[bx + nbx (by + nby bz)] = the patch
 * refining that block or -1. */
typedef struct axs_patch_map {
    const int32_t *patch_block;
    const int32_t *block_patch;
} axs_patch_map;

int axs_patches_layout(int32_t dtype, int32_t n, int32_t npatches, axs_patch_layout *out);
/* Host-synchronous: writes the device table (sweep domains, work items, tensor maps). */
int axs_patches_init(const axs_patches *p, axs_patch_plan *plan, void *stream);
/* Ghost rings (valid_too = 1: the valid cells as well) at time fraction theta
 * of the coarse step: ring cells owned by a patch are copied from it, the
 * others interpolate the coarse level -- quartic Lagrange in space, in time
 * cubic Hermite for psi (with Pi as its derivative) and linear for Pi between
 * coarse_old (start of the coarse step) and coarse_new (its end; may be NULL
 * when theta = 0). */
int axs_patches_fill(const axs_patches *p, const axs_patch_map *m, const axs_level *coarse_old,
                     const axs_level *coarse_new, double theta, double coarse_dt, int32_t valid_too, void *stream);
/* The same for the `count` patches listed in patch_list (device int32 indices;
 * entries outside [0, npatches) are skipped); NULL with count = npatches: all. */
int axs_patches_fill_list(const axs_patches *p, const axs_patch_map *m, const axs_level *coarse_old,
                          const axs_level *coarse_new, double theta, double coarse_dt, int32_t valid_too,
                          const int32_t *patch_list, int32_t count, void *stream);
/* Regrid helper: every patch box of dst (4 components, rings and padding
 * included) becomes box src_of_dst[q] of src (device int32 per dst patch), or
 * zeros where that is -1 (src may then be NULL), or is left as it is where
 * that is AXS_PATCH_KEEP. Same patch side and dtype. src and dst may share
 * their arena (same state pointer and capacity) when no box is both read and
 * written: a regrid in place moves patches from slots >= dst->npatches into
 * the free slots below it. */
#define AXS_PATCH_KEEP (-2)
int axs_patches_copy_boxes(const axs_patches *dst, const axs_patches *src, const int32_t *src_of_dst, void *stream);
/* One RK4 step of every patch (two persistent launches); the rings must hold
 * psi, Pi at time t. */
int axs_patches_rk4_step(const axs_patches *p, const axs_patch_plan *plan, const axs_background *bg, double tau_i,
                         double t, double dt, void *stream);
/* amrex::average_down: every coarse cell a patch covers becomes the mean of its
 * 8 fine children (then the coarse periodic padding is refreshed). */
int axs_patches_average_down(const axs_patches *p, const axs_patch_map *m, const axs_level *coarse, void *stream);
int axs_patches_device_status(const axs_patches *p, void *stream);
/* The fine level's part of the composite diagnostics (specific_post_timestep
 * on the finest level, AxionStringsLevel.cpp:1296-1350; count_plaquettes,
 * compute_total_energy_sums and compute_velocity_at_pierced_corners over every
 * patch, reading the rings as ghost cells): one pass over all patches, summed
 * into one result, since the patches share dx. The rings must hold the
 * snapshot's time (axs_patches_fill first). p->boundary must be
 * AXS_BOUNDARY_GHOSTS; a pierced-list entry is 4 (q n^3 + cell) + plane for
 * patch q. scratch: axs_patches_diagnostics_scratch_bytes. */
int axs_patches_diagnostics_scratch_bytes(int32_t n, int32_t npatches, int64_t *bytes);
int axs_patches_diagnostics(const axs_patches *p, const axs_diag_params *prm, axs_diag_result *out, int64_t *list,
                            int64_t capacity, void *scratch, int64_t scratch_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * Axion power spectrum (AxionStringsLevel.cpp:1583-1640): the masked a_dot
 * buffer, a caller-run unnormalised forward R2C (cuFFT), then shell binning.
 * ------------------------------------------------------------------------- */

/* fill_masked_a_dot_buffer (MaskedFieldBuffer.hpp:15-35): buf_dev[cell] =
 * masked_a_dot(psi, Pi, R) (Masking.hpp:96-118) in the level's precision,
 * dense (nz, ny, nx), x fastest; *sum_sq_dev = sum of buf^2 (MultiFab::Dot).
 * scratch: 8 bytes per block of the pass (axs_spectrum_scratch_bytes is enough). */
int axs_level_masked_a_dot(const axs_level *lv, int32_t masking_scheme, double masking_threshold, double R,
                           void *buf_dev, double *sum_sq_dev, void *scratch, int64_t scratch_bytes, void *stream);

int axs_spectrum_scratch_bytes(int32_t nx, int32_t ny, int32_t nz, int64_t *bytes);

/* compute_spectrum's binning (SpectrumKernel.hpp:77-153) of an R2C spectrum
 * spec_dev (nz, ny, nx/2+1) of interleaved complex values of `dtype`:
 * n_shells = max(nx, ny, nz)/2 + 1; shell_sum_dev[s] = sum of w 4 pi |p|^2 |X|^2
 * and shell_count_dev[s] = sum of w over modes with floor(|p| + 1/2) = s and
 * |p| < n_max/2 (w = 1 on the kx = 0 and kx = nx/2 planes, 2 elsewhere);
 * totals_dev = {full-cube energy, inscribed-sphere energy}. Deterministic. */
int axs_spectrum_bin(const void *spec_dev, int32_t dtype, int32_t nx, int32_t ny, int32_t nz, double *shell_sum_dev,
                     int64_t *shell_count_dev, double *totals_dev, void *scratch, int64_t scratch_bytes,
                     void *stream);

/* ---------------------------------------------------------------------------
 * Refinement tagging: StringTagger::operator() (StringTagger.hpp:117-151,
 * called from AxionStringsLevel::tag_cells) on a periodic level, plus the
 * buffer AMReX's TagBoxArray::buffer adds before clustering (amr.n_error_buf,
 * StringTagger.hpp:60-66) and per-block flags for fixed-size patches.
 * ------------------------------------------------------------------------- */
typedef struct axs_tag_params {
    double dx;
    double gradient_threshold;        /* dx^2 |lap psi_i| > t tags (StringTaggerParams); >= DBL_MAX: off */
    double radial_gradient_threshold; /* dx |grad |psi|| > t tags; >= DBL_MAX: off */
    int32_t n_error_buf;              /* tag every cell within this many cells (a cube, periodic) of a tag */
    int32_t block;                    /* > 0: flag each block^3 cell block that holds a tag */
} axs_tag_params;

int axs_tag_scratch_bytes(int32_t nx, int32_t ny, int32_t nz, int64_t *bytes);

/* tags_dev: nx*ny*nz bytes (cell = i + nx*(j + ny*k)), 1 = tagged.
 * block_flags_dev: ceil(nx/b)*ceil(ny/b)*ceil(nz/b) bytes when block = b > 0.
 * n_tagged_dev (nullable): number of tagged cells after buffering.
 * A cell is tagged when a plaquette at its low corner is pierced (the string
 * finder's own winding test, bit-exact), or by the two optional criteria. */
int axs_level_tag_cells(const axs_level *lv, const axs_tag_params *p, uint8_t *tags_dev, uint8_t *block_flags_dev,
                        int64_t *n_tagged_dev, void *scratch, int64_t scratch_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * Ensembles: many independent periodic boxes of uneven sizes advanced together
 * (no counterpart in the reference, which runs one box layout per process;
 * each box evolves exactly as an axs_level of its size would, bit for bit).
 *
 * The boxes are packed component-major: component c of every box lives in one
 * "component plane" of plane_elems elements; box b starts at element `base`
 * of each plane and inside it has the axs_level layout of its size (x_offset,
 * y_offset, jstride, kstride as axs_level_layout_for reports). The state arena
 * holds 4 planes, the work arena 8; both and the table are caller-owned device
 * memory, 128-byte aligned. axs_ensemble_init writes the device table (box
 * descriptors, work items, six TMA descriptor slots per box) for one tiling.
 * A two-sweep tiling runs every RK4 sweep as ONE persistent launch over the
 * work items of all boxes. The fused tiling runs every RK4 step as one launch
 * (plus one for the boxes' periodic padding), with the work arena's first 4
 * planes as the second state buffer; it takes boxes whose ny is a multiple of
 * 16 and whose nx is even. tile_config 0 is the first tiling (by id) that
 * suits every box: the fused one where it fits. After every advance the result
 * and its padding are in the state arena.
 * ------------------------------------------------------------------------- */
typedef struct axs_ensemble {
    int32_t dtype;
    int32_t nboxes;
    const int32_t *dims; /* host array, 3 per box: nx, ny, nz */
    double dx;           /* grid spacing shared by all boxes */
    void *state;         /* 4 component planes */
    void *work;          /* 8 component planes */
    void *table;         /* written by axs_ensemble_init */
    int64_t state_bytes, work_bytes, table_bytes;
} axs_ensemble;

typedef struct axs_ensemble_box {
    int64_t base;       /* element offset of the box in every component plane */
    int64_t jstride, kstride;
    int32_t x_offset, y_offset;
} axs_ensemble_box;

typedef struct axs_ensemble_plan {
    int32_t tile_config; /* in: index from axs_ensemble_tile_config_name (1..count), 0 = the first that suits */
    int32_t z_chunk;     /* in: target z planes per work item, 0 = automatic */
    int64_t n_items;     /* out: work items of one sweep (all boxes) */
    int32_t grid_a;      /* out: persistent grid of sweep A */
    int32_t grid_b;      /* out: persistent grid of sweep B */
    int64_t plane_elems; /* out */
    uint64_t key;        /* out: ties the plan to the ensemble it was built for */
} axs_ensemble_plan;

int axs_ensemble_sizes(int32_t dtype, int32_t nboxes, const int32_t *dims, int64_t *state_bytes,
                       int64_t *work_bytes, int64_t *table_bytes);
int axs_ensemble_box_layout(int32_t dtype, int32_t nboxes, const int32_t *dims, int32_t box, axs_ensemble_box *out);
int32_t axs_ensemble_tile_config_count(int32_t dtype);
const char *axs_ensemble_tile_config_name(int32_t dtype, int32_t id);

/* Build the device table for plan->tile_config / plan->z_chunk and fill the
 * plan's outputs. Host-synchronous (it uploads the table and waits); call it
 * before capturing axs_ensemble_rk4_advance in a CUDA graph. */
int axs_ensemble_init(const axs_ensemble *e, axs_ensemble_plan *plan, void *stream);

/* Periodic padding of every box (after the caller wrote the valid cells). */
int axs_ensemble_fill_ghosts(const axs_ensemble *e, void *stream);

/* nsteps classic-RK4 steps of every box: two persistent launches per step
 * (sweeps A and B over all boxes' work items). Graph-capturable. The plan must
 * be the one the last axs_ensemble_init on this table returned (checked on the
 * host; a stale plan is rejected with AXS_ERR_INVALID_ARGUMENT). */
int axs_ensemble_rk4_advance(const axs_ensemble *e, const axs_ensemble_plan *plan, const axs_background *bg,
                             double tau_i, double t0, double dt, int32_t nsteps, void *stream);

/* Per-box diagnostics (as axs_level_diagnostics, without the pierced list)
 * into result_dev[0 .. nboxes-1]. The boxes run on up to 8 internal streams
 * side by side, forked from and joined back to `stream` with events (parallel
 * branches under graph capture); scratch, sized by
 * axs_ensemble_diagnostics_scratch_bytes, holds one slice per stream. The
 * internal streams are created on a device's first call and kept for the life
 * of the process: do not call it again after a cudaDeviceReset of that device. */
int axs_ensemble_diagnostics_scratch_bytes(int32_t nboxes, const int32_t *dims, int64_t *bytes);
int axs_ensemble_diagnostics(const axs_ensemble *e, const axs_diag_params *p, axs_diag_result *result_dev,
                             void *scratch, int64_t scratch_bytes, void *stream);

/* Host-synchronous: AXS_ERR_DEVICE_TIMEOUT if a sweep's bounded wait gave up. */
int axs_ensemble_device_status(const axs_ensemble *e, void *stream);

/* ---------------------------------------------------------------------------
 * Initial data
 * ------------------------------------------------------------------------- */

/* FourierIC::generate's spectral fill (FourierIC.hpp:82-116) on the device:
 * the R2C half spectrum (nz, ny, nx/2+1) of interleaved (re, im) doubles with
 * hash-seeded Gaussian modes for 0 < k^2 <= k_max_cells^2. The inverse real
 * FFT and the rescale to the target mean square follow on the caller's side. */
int axs_fourier_spectrum(double *spec_dev, int32_t nx, int32_t ny, int32_t nz, double k_max_cells,
                         uint64_t seed, int32_t comp_seed_offset, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* AXS_H */
