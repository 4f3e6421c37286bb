/*
 * palgpu.h -- C ABI of the GB300-native palinstrophy DNS step (libpalgpu.so).
 *
 * The reference has no FFI of its own: its "operator API" is the set of Python
 * functions in palinstrophy/turbo_simulator.py that the sim CLI (run_dns) and
 * the GUI facade (turbo_wrapper.py DnsSimulator) call, plus the DnsState
 * fields they read.  Each entry point below replaces one of those functions
 * (file:line cited beside it); palinstrophy_gb300/turbo_simulator.py binds
 * them with ctypes and re-exports the reference's Python names.
 *
 * Conventions
 *   - Every call returns an int status: PAL_OK (0) or a negative PAL_ERR_*;
 *     pal_last_error() gives the message.  No exception crosses the ABI.
 *   - One handle = one field on the current CUDA device, with its own stream;
 *     a handle is used from one host thread at a time.
 *   - Host arrays are in the reference layouts and in the handle's precision:
 *     complex64 (interleaved float re, im) for PAL_FP32, complex128 for PAL_FP64.
 *       om2, fnm1 : (N, N/2)     [z][kx]
 *       uc_low    : (2, N, N/2)  [comp][z][kx]  (uc_full[0:2, :N, :N/2])
 *       ur planes : (M, M) real  [z][x], M = 3N/2
 *   - Step calls are asynchronous on the handle's stream; only pal_get_* ,
 *     pal_compute_cflm, pal_diagnostics and pal_synchronize wait for it.
 */
#ifndef PALGPU_H
#define PALGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PAL_OK = 0,
  PAL_ERR_INVALID = -1,     /* bad argument (null handle/pointer, unsupported N, ...) */
  PAL_ERR_CUDA = -2,        /* a CUDA runtime call failed */
  PAL_ERR_OOM = -3,         /* device allocation failed */
  PAL_ERR_STATE = -4,       /* call out of order (e.g. step3 before step2b) */
  PAL_ERR_NONFINITE = -5,   /* NaN/Inf detected in the field */
  PAL_ERR_TIMEOUT = -6      /* a kernel's bounded wait for its own bulk copies ran out (reported by the
                               next call that reads the device scalars, which clears it) */
};

enum { PAL_FP32 = 0, PAL_FP64 = 1 };
enum { PAL_CNAB2 = 0, PAL_LS_IMEX_RK3 = 1 };
enum { PAL_FIELD_OM2 = 0, PAL_FIELD_FNM1 = 1, PAL_FIELD_UR_U = 2, PAL_FIELD_UR_V = 3 };
enum { PAL_SPEC_KM3 = 0, PAL_SPEC_PAO = 1 };
enum { PAL_VAR_U = 0, PAL_VAR_V = 1, PAL_VAR_ENERGY = 2, PAL_VAR_OMEGA = 3, PAL_VAR_STREAM = 4 };
enum { PAL_SC_T = 0, PAL_SC_DT = 1, PAL_SC_CN = 2, PAL_SC_CNM1 = 3, PAL_SC_VISC = 4, PAL_SC_CFLNUM = 5, PAL_SC_IT = 6 };

typedef struct pal_handle pal_handle;

/* Diagnostics, all FP64 (turbo_simulator.py:764-810, turbo_main.py:1947-1959, 2015-2073). */
typedef struct pal_diag {
  double U;                  /* sqrt(mean(u^2 + v^2)) on the 3/2 grid */
  double L;                  /* 2 pi sum(w |om|^2/K^3) / E */
  double tau_l;              /* L / U */
  double E;                  /* sum over K2>0 of w |om|^2 / K2 */
  double Z;                  /* enstrophy sum: sum w |om|^2 - |om_00|^2 */
  double P;                  /* palinstrophy sum: sum w K2 |om|^2 */
  double kmax2;              /* max K2 of the compact band */
  double pal_over_ens_kmax2; /* P / (Z kmax2), the GUI metric */
  double cflm;               /* max(|u|+|v|) N/(2 pi) */
  double energy_joules;      /* 0.5 (2 pi)^2 mean(u^2+v^2) */
  int nonfinite;             /* 1 if a NaN/Inf was seen */
} pal_diag;

/* create_dns_state (turbo_simulator.py:878-1054): allocate the device state for
 * an N x N field (N in 32..8192, see pal_supported).  visc defaults to
 * float32(1/Re) as dns_pao_host_init sets it (turbo_simulator.py:470, 1139);
 * cfl is the CFL target cflnum.  The state is empty until pal_set_* calls. */
int pal_create(int N, int precision, double Re, double cfl, pal_handle** out);
int pal_destroy(pal_handle* h);
/* 1 if (N, precision) has compiled kernels, else 0. */
int pal_supported(int N, int precision);
/* Device properties of the handle's GPU: SM count and max dynamic smem per block. */
int pal_device_info(int* sm_count, int* smem_optin, char* name, size_t name_len);

/* Initial state as create_dns_state leaves it (turbo_simulator.py:1191-1234):
 * om2 and fnm1 (fnm1 may be NULL for zeros), and the velocity low band that
 * the first dns_step2a transforms (uc_low may be NULL: then the velocity is
 * rebuilt from om2 by the inversion of turbo_simulator.py:1555-1585).  The
 * arrays may be in host or device memory (copied with unified addressing). */
int pal_set_spectral_state(pal_handle* h, const void* om2, const void* fnm1);
int pal_set_velocity_spectrum(pal_handle* h, const void* uc_low);

/* DnsState scalar mirror (turbo_simulator.py:742-753, 846-854). */
int pal_set_scalars(pal_handle* h, double t, double dt, double cn, double cnm1, double visc,
                    double cflnum, long long it);
int pal_get_scalars(pal_handle* h, double* t, double* dt, double* cn, double* cnm1, double* visc,
                    double* cflnum, long long* it);
/* One scalar (PAL_SC_*), as DnsState.__setattr__ mirrors dt/cn/cnm1 into the
 * device time_scalars (turbo_simulator.py:742-753); stream-ordered. */
int pal_set_scalar(pal_handle* h, int which, double value);

/* dns_step2a (turbo_simulator.py:1949-2100): pad + inverse transform of the
 * velocity spectrum.  After pal_step3 the column half is already done by the
 * fused column kernel, so this only completes a pending initial transform. */
int pal_step2a(pal_handle* h);
/* dns_step2b (turbo_simulator.py:1378-1513): products + forward transform
 * (the x half; the z half is fused into pal_step3). */
int pal_step2b(pal_handle* h);
/* dns_step3 (turbo_simulator.py:1588-1771): nonlinear term, CNAB2 update,
 * fnm1 <- fn, cnm1 <- cn, omega -> velocity inversion (+ the z half of the next
 * dns_step2a). */
int pal_step3(pal_handle* h);
/* dns_step_ls_imex_rk3 (turbo_simulator.py:1900-1943): one full 3-stage step. */
int pal_step_rk3(pal_handle* h);
/* The run_dns hot loop (turbo_simulator.py:2831-2848) for nsteps steps of
 * `method`: after the step with iteration number it (counted by the handle),
 * NEXTDT runs if update > 0 and (it % update == 0 || it == 1 || (final_update
 * && last step of this call)); t += dt_old and it += 1 every step. */
int pal_step(pal_handle* h, int method, int nsteps, int update, int final_update);

/* compute_cflm (turbo_simulator.py:2106-2125), waits for the result. */
int pal_compute_cflm(pal_handle* h, double* cflm);
/* next_dt (turbo_simulator.py:2127-2167): CFLM, cn = 0.8 + 0.2 cflnum/CFL,
 * dt *= cn on the device.  With sync_host != 0 it waits and stores CFLM. */
int pal_next_dt(pal_handle* h, int sync_host, double* cflm);
/* flow_eddy_metrics + the GUI sums in one pass; waits. */
int pal_diagnostics(pal_handle* h, pal_diag* out);

/* Shell-binned kinetic-energy spectrum from om2 (compute_energy_spectrum_uv_bins,
 * turbo_simulator.py:2225-2383): nbins bins of r = |k|/k_nyq over [0, r_max),
 * esum[b] = sum |om|^2/K2 * (M^2)^2 (x2 for kx > 0), count[b] = modes (x2 for
 * kx > 0); deterministic; waits. */
int pal_energy_spectrum(pal_handle* h, int nbins, double r_max, double k_nyq, double* esum, int* count);

/* Display fields of DnsSimulator (turbo_wrapper.py:353-413, turbo_simulator.py:
 * 2629-2709) on the 3/2 grid, M x M: u, v, |u| (dns_kinetic), omega
 * (dns_om2_phys) or the streamfunction (dns_stream_func), into host_field
 * (real, handle precision) and/or host_pixels (uint8, normalised to 1..255,
 * 128 if constant, as _float_to_pixels_gpu).  Uses separate scratch planes,
 * so the simulation state is unchanged.  Waits. */
int pal_vis_field(pal_handle* h, int var, void* host_field, unsigned char* host_pixels);

/* Gradient of the final palinstrophy L = 1/2 sum w' K2 |om|^2 (w' = 1 for kx = 0,
 * else 2: 1/2 <|grad omega|^2> on the grid) after nsteps LS-IMEX-RK3 steps at
 * the handle's fixed dt (no NEXTDT), with respect to the current om2 (the
 * velocity is taken as its inversion).  Hand-written discrete adjoint of the
 * stage (transposed padded transforms, adjoint products and inversion, reversed
 * IMEX stages), states checkpointed every ckpt_every steps and recomputed.
 * grad_host receives dL/d(om2) in the reference layout (real inner product
 * Re sum conj(g) d om2); the handle ends at the final forward state.  The
 * reference has no differentiation; N = 32..512.  Waits. */
int pal_adjoint_palinstrophy(pal_handle* h, int nsteps, int ckpt_every, double* loss, void* grad_host);

/* Copy a field to host memory in the reference layout (waits). */
int pal_get_field(pal_handle* h, int which, void* host_dst);
/* Device pointer of a field: om2/fnm1 are stored transposed, [kx][z] (N/2 x N);
 * the physical planes [z][x] are valid after pal_get_field(UR_U/UR_V) or
 * pal_materialize_physical. */
int pal_field_device_ptr(pal_handle* h, int which, void** ptr);
int pal_materialize_physical(pal_handle* h);
int pal_synchronize(pal_handle* h);
/* Per-kernel timing: runs nsteps steps of `method` (no NEXTDT) with a CUDA
 * event between consecutive launches on the handle's stream and returns the
 * average duration of the row pass (k_row) and of the column pass (k_col) in
 * milliseconds, and the number of kernels launched.  Measurement support; no
 * counterpart in the reference. */
int pal_profile_kernels(pal_handle* h, int method, int nsteps, double* ms_row, double* ms_col, int* launches);
/* FP64 FMA throughput of the current GPU in TFLOP/s (best of 5 timed launches of
 * an FMA-chain kernel filling every SM, CUDA events; *ms = that launch's time):
 * the ceiling of the FP64 plain path, whose kernels are bound by the FP64 pipe.
 * Measurement support; no counterpart in the reference. */
int pal_fp64_peak(double* tflops, double* ms);
/* Kernel candidates: for each N the library compiles several row-pass and
 * column-pass kernels (radix order, rows per tile, threads per block).
 * pal_create times them on the new handle and keeps the fastest, once per
 * (precision, N) per process; PAL_AUTOTUNE=0 in the environment keeps the
 * first candidates instead, and PAL_TMA_MULTICAST=0 leaves out the candidates
 * that load by TMA cluster multicast (N=8192 "... mc ...").  With
 * PAL_TUNE_FILE=<path>, a size listed in that file
 * ("fp32 <N> <row name>|<column name>" per line) takes the named candidates
 * without timing and a timed size is appended, so that later processes run
 * the same kernels.  pal_get_variant reports the choice and a short
 * description; pal_set_variant forces one (between steps).  Performance
 * control; no counterpart in the reference. */
int pal_get_variant(pal_handle* h, int* row, int* col, int* n_rows, int* n_cols, char* desc, size_t desc_len);
int pal_set_variant(pal_handle* h, int row, int col);
/* Resident blocks per SM of the selected row and column kernels, from the CUDA
 * occupancy calculator (diagnostic; no counterpart in the reference). */
int pal_get_occupancy(pal_handle* h, int* row_blocks_per_sm, int* col_blocks_per_sm);
/* Test switches (no counterpart in the reference).  PAL_DBG_SKIP_FIRST_WAIT,
 * value 1: the kernels that move tiles by TMA give their first wait for the
 * tile's bulk copies no polls, so they take the path that reports a timed-out
 * wait (PAL_ERR_TIMEOUT from the next pal_get_scalars / pal_compute_cflm /
 * pal_diagnostics), then wait for the copies with the normal bound before using
 * the tile; the results stay valid.  Value 0 restores the normal waits. */
enum { PAL_DBG_SKIP_FIRST_WAIT = 0 };
int pal_set_debug(pal_handle* h, int what, int value);
/* The handle's CUDA stream (cudaStream_t), for event timing or interop. */
int pal_get_stream(pal_handle* h, void** stream);
int pal_last_error(pal_handle* h, char* buf, size_t n);

/* Allocation-free stepping for callers that cannot allocate device memory at
 * the point of the call (inside host callbacks or real-time loops that must not
 * block on the allocator, plugins whose host forbids device allocations after
 * start-up, tools that budget device memory up front).  No counterpart in the
 * reference.  Advances a field given as caller-owned device arrays om2 and
 * fnm1 ((N, N/2) complex64, reference layout, updated in place) by nsteps steps
 * of `method` at fixed dt (no NEXTDT), with the velocity rebuilt from om2 first
 * and cn/cnm1 the AB2 weights of the first CNAB2 step.  Work planes live in a
 * 6 MiB scratch array inside the library (one per GPU, resident until exit):
 * FP32 only and N <= 512, otherwise PAL_ERR_INVALID.  Nothing is allocated.
 * Asynchronous on `stream`; calls whose GPU work overlaps share the scratch
 * and race.  The first call on a device looks the scratch up and should come
 * before any stream capture. */
int pal_step_noalloc(int N, int method, int nsteps, double dt, double visc, double cn, double cnm1,
                     void* om2, void* fnm1, void* stream);

/* Batched ensembles (the reference runs one field per process; this is the
 * GB300 form for many independent fields): members with their own N, seed,
 * viscosity, CFL target and adaptive dt advance together, optionally replayed
 * from a CUDA graph.  When every member's N belongs to a compiled fused set
 * (FP32: N = 256, 384, 512) each pass is ONE launch over all members of all
 * sizes (2 launches per CNAB2 step, 6 per LS-IMEX-RK3 step); otherwise, or
 * with PAL_ENSEMBLE_FUSED=0 in the environment, one launch per group of equal
 * N per pass (grid.y = members).  No counterpart in the reference API; each
 * member follows the single-field semantics of pal_step. */
typedef struct pal_ensemble pal_ensemble;
int pal_ensemble_create(int n_members, const int* N, int precision, double Re, double cfl, pal_ensemble** out);
int pal_ensemble_destroy(pal_ensemble* e);
/* Member state in the reference layouts (as pal_set_spectral_state +
 * pal_set_velocity_spectrum); fnm1 / uc_low may be NULL. */
int pal_ensemble_set_member(pal_ensemble* e, int member, const void* om2, const void* fnm1, const void* uc_low);
/* One scalar (PAL_SC_*) of one member, or of all members with member = -1. */
int pal_ensemble_set_scalar(pal_ensemble* e, int member, int which, double value);
/* Initial STEP2A + CFLM + dt = cflnum/(CFLM pi), cn = 1, cnm1 = 0 per member
 * (turbo_simulator.py:2810-2823), on the device. */
int pal_ensemble_init_dt(pal_ensemble* e);
/* nsteps steps of every member with NEXTDT per member after iterations
 * it % update == 0 or it == 1 (update > 0); use_graph captures the launch
 * sequence once per pattern and replays it. */
int pal_ensemble_step(pal_ensemble* e, int method, int nsteps, int update, int use_graph);
/* Re-tune each group's row / column candidates on its batched launch shape and
 * run per-size launches of them; call right after pal_ensemble_create, before
 * any member is set.  Without it the groups use the fused set's candidates or
 * the single-field choice of pal_create (members then match single fields of
 * those candidates bit for bit; tuned groups match them to rounding). */
int pal_ensemble_autotune(pal_ensemble* e);
/* Candidates of the group of size group_N, as "row[...] col[...]". */
int pal_ensemble_get_variant(pal_ensemble* e, int group_N, char* desc, size_t desc_len);
int pal_ensemble_get_member(pal_ensemble* e, int member, int which, void* host_dst);
int pal_ensemble_get_scalars(pal_ensemble* e, int member, double* t, double* dt, double* cn, double* cflm,
                             long long* it);
int pal_ensemble_get_stream(pal_ensemble* e, void** stream);
int pal_ensemble_synchronize(pal_ensemble* e);
int pal_ensemble_last_error(pal_ensemble* e, char* buf, size_t n);

/* PAO / KM3 initial condition generated into the handle (turbo_simulator.py:
 * 213-485, 1059-1239, 1314-1361): the LCG draws run on the host in the
 * reference's serial order, the per-mode PAO amplitudes and phases, the KM3
 * shell sums and rescale, the moments and om2 = i (gamma u1 - alfa u3) on the
 * device.  Sets om2, the velocity band (as pal_set_velocity_spectrum) and
 * fnm1 = 0; uc_host, if not null, receives the velocity band (2, N, N/2) in the
 * handle's precision.  stats[0..2] = Energy, WiWi, visc; *seed_out = final LCG
 * seed.  Replaces the host-side generator call of create_dns_state.  Waits. */
int pal_generate(pal_handle* h, double K0, double Re, int seed, int spectrum, void* uc_host, double* stats,
                 int* seed_out);

/* Host-side PAO / KM3 initial condition (turbo_simulator.py:213-485, 1059-1239,
 * 1314-1361), complex64 outputs: om2 (N, N/2) and uc_low (2, N, N/2).
 * stats[0..2] = Energy (Q2), WiWi (W2), visc; *seed_out = final LCG seed.
 * The per-mode float32 cos/sin/exp come from the C library here; the reference
 * takes them from NumPy's float32 ufuncs, which can differ in the last bit. */
int pal_pao_generate(int N, double K0, double Re, int seed, int spectrum, void* om2, void* uc_low,
                     double* stats, int* seed_out);
/* The generator in two halves around its three float32 transcendental values,
 * so that a caller can evaluate those with the reference's own functions
 * (NumPy's float32 ufuncs) and reproduce the reference's arrays bit for bit.
 * pal_pao_draws: the serial LCG + 97-entry shuffle of turbo_simulator.py:241-286;
 * v[z * N/2 + x] = the shuffled variate of mode (x, z) in the reference's call
 * order, *seed_out = final LCG seed.
 * pal_pao_build: turbo_simulator.py:287-470 and 1314-1361 from
 * cos_th = cos(2 pi v), sin_th = sin(2 pi v) (2 pi v formed as
 * (float(2) * float(pi)) * v) and exp_g = exp(-(k/K0)^2) (k = sqrt(float(kx^2 +
 * kz^2)), -(k/K0) * (k/K0) in float), all float32 in the layout of v; outputs as
 * pal_pao_generate. */
int pal_pao_draws(int N, int seed, float* v, int* seed_out);
int pal_pao_build(int N, double K0, double Re, int seed, int spectrum, const float* cos_th, const float* sin_th,
                  const float* exp_g, void* om2, void* uc_low, double* stats);

#ifdef __cplusplus
}
#endif
#endif /* PALGPU_H */
