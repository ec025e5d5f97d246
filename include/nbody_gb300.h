/*
 * nbody_gb300.h -- C ABI of the GB300 (sm_103a) all-pairs gravity library.
 *
 * Plain pointers and sizes only.  Streams are passed as `void *` holding a
 * cudaStream_t (NULL = the legacy default stream).  Device pointers must be
 * 16-byte aligned (float4 arrays); workspaces 256-byte aligned.
 *
 * Layouts follow the reference (src/nbody.cu:127-156):
 *   posMass     float4 {x, y, z, m}
 *   velInvMass  float4 {vx, vy, vz, 1/m}
 *   force       float4 {fx, fy, fz, w}; the sum carries m_j but not m_i or G,
 *               i.e. it is the acceleration (src/bodybodyInteraction.cuh:40-65)
 */
#ifndef NBODY_GB300_H
#define NBODY_GB300_H

#include <stddef.h>

#include "nbgb_status.h"

#define NBGB_API __attribute__((visibility("default")))

#ifdef __cplusplus
extern "C" {
#endif

/* ======================================================================== */
/* Drop-in algorithm entry point                                             */
/* ======================================================================== */

/*
 * Replaces: pfnComputeGravitation_AOS_t (src/nbody.h:68), i.e. one more row
 * of s_algorithms[] (src/nbody.cu:83-103) of type ALGORITHM_AOS_GPU, like
 * ComputeGravitation_GPU_Shared (src/nbody_GPU_Shared.cu:83-103).
 *
 * force, posMass: DEVICE pointers to N float4 each (the driver's
 * g_dptrAOS_Force / g_dptrAOS_PosMass, src/nbody.cu:351-370).  Writes
 * force[i].xyz and sets force[i].w = 0.  Any N >= 1 is accepted (the
 * reference driver always passes a multiple of 1024).
 *
 * Runs on the legacy default stream, synchronises the device before
 * returning, and returns the elapsed milliseconds measured by CUDA events
 * around its launches; returns 0 on any error, which the reference driver
 * treats as "skip this algorithm" (src/nbody.cu:385-386).  Scratch space is
 * allocated on first use and cached per device (nbgb_release_workspace frees
 * it).  Not re-entrant across host threads on the same device.  Masses may
 * have any sign: when the planner's configuration takes source pairs in the
 * log domain (below) and meets a negative mass, the call evaluates again with
 * rsqrt-only arithmetic and times that evaluation.
 */
NBGB_API float ComputeGravitation_GPU_GB300(float *force, float *posMass, float softeningSquared,
                                            size_t N);

/* A second row for the table, same signature and conventions: the
   Newton's-third-law variant (nbgb_force_newton3), each pair evaluated once;
   like the reference's unregistered tiled kernels
   (src/nbody_GPU_AOS_tiled.cu:181-218). */
NBGB_API float ComputeGravitation_GPU_GB300_Newton3(float *force, float *posMass,
                                                    float softeningSquared, size_t N);

/* Frees the drop-in entry point's cached scratch space on every device.
   Scratch cached in a context that has since been reset (cudaDeviceReset)
   is forgotten, not freed: the reset released it, and the next call
   allocates afresh. */
NBGB_API void nbgb_release_workspace(void);

/* ======================================================================== */
/* Stream-ordered force evaluation with a caller-owned workspace             */
/* ======================================================================== */

/* Workspace bytes nbgb_force needs for N bodies on the current device
   (0 if N is unsupported). */
NBGB_API size_t nbgb_force_workspace_bytes(size_t N);

/*
 * Same sum as ComputeGravitation_GPU_GB300 (replaces the kernel launch inside
 * the reference's GPU algorithms, e.g. src/nbody_GPU_Shared.cu:91-95), but
 * asynchronous on `stream`, with scratch in a caller-provided DEVICE
 * workspace of at least nbgb_force_workspace_bytes(N) bytes.  Returns
 * NBGB_OK or a negative NBGB_ERR_* code; device-side failures are reported by
 * nbgb_last_status after the stream is synchronised.  Calls that share a
 * workspace must not overlap on the GPU.
 *
 * Masses: the planner's default configurations (names ending in "log4") take
 * every fourth source pair's m r^-3 as 2^(log2 m - 1.5 log2 r^2), which needs
 * m >= 0.  A negative (or NaN) mass gives NaN forces and sets
 * NBGB_STATUS_NEGATIVE_MASS; for signed masses force an rsqrt-only
 * configuration through nbgb_force_ex.
 */
NBGB_API int nbgb_force(float *force, const float *posMass, float softeningSquared, size_t N,
                        void *workspace, size_t workspace_bytes, void *stream);

/* As nbgb_force with the kernel configuration and j-split forced.  config:
   -1 the planner's choice.  nsplit: -1 the planner's choice; > 0 every
   i-block's j-range split nsplit ways; <= -2 whole i-blocks for the whole
   rounds of CTA slots they fill and only the leftover i-blocks split
   -nsplit ways (every i-block, when they fill no whole round).  For tests
   and tuning. */
NBGB_API int nbgb_force_ex(float *force, const float *posMass, float softeningSquared, size_t N,
                           void *workspace, size_t workspace_bytes, int config, int nsplit,
                           void *stream);

/*
 * Newton's-third-law variant (the reference's unregistered tiled kernels,
 * src/nbody_GPU_AOS_tiled.cu:93-179, compute each pair once too): each pair
 * is evaluated once and applied to both bodies; per-block-pair sums are
 * accumulated in FP64 and rounded to FP32 at the end.  Same arguments and
 * conventions as nbgb_force; workspace >= nbgb_force_newton3_workspace_bytes.
 */
/*
 * Replaces: one GPU's share of the reference's multi-GPU algorithm
 * (ComputeGravitation_multiGPU / ComputeNBodyGravitation_multiGPU,
 * src/nbody_multiGPU.cu:47-125): the forces on target rows
 * [row_begin, row_end) of posMass against all N sources.  posMass: DEVICE,
 * all N bodies (replicated on every GPU, as the reference copies it to
 * each); force_rows: DEVICE float4[row_end - row_begin].  Unlike the
 * reference, any split of the rows is accepted (it requires N % GPUs == 0).
 * Workspace: nbgb_force_rows_workspace_bytes(N, rows), 256-byte aligned.
 * Stream-ordered.  nbody_gb300.sharded drives one rank per GPU with it.
 */
NBGB_API size_t nbgb_force_rows_workspace_bytes(size_t N, size_t rows);
NBGB_API int nbgb_force_rows(float *force_rows, const float *posMass, float softeningSquared,
                             size_t N, size_t row_begin, size_t row_end, void *workspace,
                             size_t workspace_bytes, void *stream);

NBGB_API size_t nbgb_force_newton3_workspace_bytes(size_t N);
NBGB_API int nbgb_force_newton3(float *force, const float *posMass, float softeningSquared,
                                size_t N, void *workspace, size_t workspace_bytes, void *stream);

/* The planner's decision for N (config forced when >= 0, nsplit as for
   nbgb_force_ex). */
NBGB_API int nbgb_force_plan(size_t N, int config, int nsplit, int *out_config, int *out_nsplit,
                             size_t *out_workspace_bytes);
/* The same decision without a GPU, for a device with `sms` SMs and
   occupancy[c] resident CTAs per SM of configuration c (nconfigs must equal
   nbgb_force_num_configs()); out_nfull: i-blocks kept whole. */
NBGB_API int nbgb_force_plan_on(size_t N, int sms, const int *occupancy, int nconfigs, int config,
                                int nsplit, int *out_config, int *out_nsplit, int *out_nfull,
                                size_t *out_workspace_bytes);
/* The current device's SM count and resident CTAs per SM of every
   configuration, as the planner uses them (nconfigs >= the number). */
NBGB_API int nbgb_force_device_info(int *sms, int *occupancy, int nconfigs);
NBGB_API int nbgb_force_num_configs(void);
NBGB_API const char *nbgb_force_config_name(int config);
/* Relative throughput the planner assumes for a configuration (measured
   defaults); an autotuner sets measured values.  Not thread-safe against
   concurrent planning. */
NBGB_API int nbgb_force_set_speed(int config, double speed);
NBGB_API double nbgb_force_get_speed(int config);

/*
 * Allocation-free force evaluation.  No counterpart in the reference: it is
 * for callers that cannot call cudaMalloc at run time -- hosts that own all
 * device memory through their own pool or a budget fixed at start-up, and
 * latency-critical step loops, where cudaMalloc/cudaFree may synchronise the
 * device and take driver-wide locks.  Same sum and arguments as nbgb_force,
 * but the scratch space is a fixed 32 MiB device array inside the library
 * (held on every GPU that loads the library until the process exits), so
 * nothing is allocated.  N is limited to 2,097,152 bodies; larger N returns
 * NBGB_ERR_TOO_LARGE without launching anything.  All calls on a device share
 * the array: calls that overlap on the GPU race.  The first call on a device
 * looks up the array's address (once per device); make it before capturing
 * any stream.  Asynchronous on `stream`; returns NBGB_OK or NBGB_ERR_*.
 * Masses >= 0, as for nbgb_force with the planner's choice.
 */
NBGB_API int nbgb_force_static(float *force, const float *posMass, float softeningSquared,
                               size_t N, void *stream);
/* Size of that fixed scratch array in bytes. */
NBGB_API size_t nbgb_force_static_capacity_bytes(void);

/* ======================================================================== */
/* Integration step                                                          */
/* ======================================================================== */

/*
 * Replaces: integrateGravitation_SOA / integrateOne (src/nbody.cu:158-236),
 * which the reference runs on one host thread.  DEVICE float4 arrays, in
 * place: v += (F * invMass) * dt; v *= damping; x += v * dt, each operation
 * rounded separately in binary32 (bit-identical to IEEE single precision
 * evaluation of that formula on the host).  posMass.w and velInvMass.w are
 * preserved.  Asynchronous on `stream`.
 */
NBGB_API int nbgb_integrate_reference(float *posMass, float *velInvMass, const float *force,
                                      float dt, float damping, size_t N, void *stream);

/*
 * Replaces: the same step as the reference binary computes it.  Built with
 * its own flags (meson.build:33-38: -O3 -ffast-math -march=native), GCC
 * contracts the position update of integrateOne (src/nbody.cu:178-181) into
 * one fused multiply-add and keeps the velocity update as written.
 * fused_drift = 1 reproduces that (x = fma(v, dt, x)), bit-identical to the
 * reference's compiled integrateGravitation_SOA; fused_drift = 0 is
 * nbgb_integrate_reference.
 */
NBGB_API int nbgb_integrate_reference_ex(float *posMass, float *velInvMass, const float *force,
                                         float dt, float damping, size_t N, int fused_drift,
                                         void *stream);

/* ======================================================================== */
/* Device-resident simulation (the reference's per-step orchestration,      */
/* src/nbody.cu:293-470, without host copies)                               */
/* ======================================================================== */

#define NBGB_INTEGRATOR_REFERENCE 0       /* integrateOne, FP32, damping       */
#define NBGB_INTEGRATOR_KDK64 1           /* FP64 kick-drift-kick, a = F        */
#define NBGB_INTEGRATOR_REFERENCE_FUSED 2 /* integrateOne with x = fma(v,dt,x),
                                             as the reference binary computes */

typedef struct nbgb_system nbgb_system;

/* Allocates all device state on the current device; NULL on failure.  A
   system (and an ensemble, below) belongs to the CUDA context it was created
   in: destroy it before a cudaDeviceReset. */
NBGB_API nbgb_system *nbgb_system_create(size_t N, int integrator, float softeningSquared,
                                         float dt, float damping);
NBGB_API void nbgb_system_destroy(nbgb_system *sys);
/* HOST float4 arrays in (posMass, velInvMass).  A mass < 0 moves the
   system onto an rsqrt-only force configuration (see nbgb_force). */
NBGB_API int nbgb_system_set_state(nbgb_system *sys, const float *posMass,
                                   const float *velInvMass);
/* KDK only: HOST double[N][3] positions and velocities, float[N] masses. */
NBGB_API int nbgb_system_set_state64(nbgb_system *sys, const double *pos3, const double *vel3,
                                     const float *mass);
/* Advance nsteps (asynchronous; whole groups of 8 steps replay a captured
   CUDA graph, the rest launch directly).  Reference integrators with the
   one-sided kernel: each step is one launch (the force kernel integrates
   each body in its epilogue).  KDK: each step is one kick+drift launch and
   one force launch; the call's closing half kick is applied when the
   velocities are next read (getters, diagnostics) or merged into the next
   call's opening kick. */
NBGB_API int nbgb_system_step(nbgb_system *sys, int nsteps);
/* KDK: apply a pending closing half kick now (asynchronous). */
NBGB_API int nbgb_system_sync_velocities(nbgb_system *sys);
NBGB_API int nbgb_system_set_graph(nbgb_system *sys, int enable);
/* 0: one-sided force kernel (default); 1: Newton's-third-law variant. */
NBGB_API int nbgb_system_set_force_algorithm(nbgb_system *sys, int algorithm);
/* Bracket every force launch and every integrate launch with CUDA events on
   the system's stream (steps then run eagerly); nbgb_system_last_force_ms
   reads the latest force launch, nbgb_system_last_integrate_ms the latest
   integrate launches: step_ms the reference integrate or the FP64
   kick+drift, half_kick_ms the closing FP64 half kick (0 if none ran).  With
   a reference integrator and the one-sided kernel the integrate runs inside
   the force launch (its epilogue), so the force time covers both and
   nbgb_system_last_integrate_ms has nothing to report (-1). */
NBGB_API int nbgb_system_set_timing(nbgb_system *sys, int enable);
NBGB_API int nbgb_system_last_force_ms(nbgb_system *sys, float *ms);
NBGB_API int nbgb_system_last_integrate_ms(nbgb_system *sys, float *step_ms,
                                           float *half_kick_ms);
NBGB_API int nbgb_system_synchronize(nbgb_system *sys);
/* HOST float4 arrays out (either may be NULL); synchronises. */
NBGB_API int nbgb_system_get_state(nbgb_system *sys, float *posMass, float *velInvMass);
NBGB_API int nbgb_system_get_state64(nbgb_system *sys, double *pos3, double *vel3);
/* Forces of the most recent force pass, HOST float4; synchronises. */
NBGB_API int nbgb_system_get_force(nbgb_system *sys, float *force);
/* Conserved quantities at the current state in FP64: out[0] kinetic,
   out[1] potential energy (softened, self pairs excluded), out[2..4] linear
   and out[5..7] angular momentum.  Costs one extra all-pairs pass (force
   kernel with the potential); synchronises. */
NBGB_API int nbgb_system_diagnostics(nbgb_system *sys, double *out);
NBGB_API void *nbgb_system_device_posmass(nbgb_system *sys);
NBGB_API void *nbgb_system_device_force(nbgb_system *sys);
NBGB_API void *nbgb_system_stream(nbgb_system *sys);
NBGB_API int nbgb_system_plan(nbgb_system *sys, int *config, int *nsplit);
/* Force the one-sided kernel's plan (config / nsplit as for nbgb_force_ex;
   -1, -1 restores the planner's choice).  For tuning and tests; the
   potential configuration is refused, log-domain configurations need
   masses >= 0.  Synchronises the system's stream. */
NBGB_API int nbgb_system_set_plan(nbgb_system *sys, int config, int nsplit);

/* ======================================================================== */
/* Ensembles of independent systems (batched and served)                     */
/* ======================================================================== */

/* No counterpart in the reference (it evaluates one system per call,
   src/nbody.h:68).  All active systems live in one device arena; a tick
   advances every one by an FP64 kick-drift-kick step with three launches, the
   force pass being ONE persistent launch over a device queue of (system,
   i-block, j-split) work items.  A system's plan depends only on its N, so
   results are bit-identical alone or in any mix.  Host calls on one ensemble
   must come from one thread. */
typedef struct nbgb_ensemble nbgb_ensemble;

/* Allocates the whole arena for max_bodies bodies / max_systems systems;
   NULL on failure.  nbgb_ensemble_device_bytes reports its size. */
NBGB_API nbgb_ensemble *nbgb_ensemble_create(size_t max_bodies, int max_systems,
                                             float softeningSquared);
NBGB_API void nbgb_ensemble_destroy(nbgb_ensemble *ens);
NBGB_API size_t nbgb_ensemble_device_bytes(nbgb_ensemble *ens);
/* Plan for N in [2^bucket, 2^(bucket+1)): variant 0..3 = (targets per
   thread, unroll) (1,8) (2,4) (1,4) (2,8); tile a power of two in 16..1024
   bodies; j-split 1..4; variant -1 = the default rule. */
NBGB_API int nbgb_ensemble_set_bucket_plan(nbgb_ensemble *ens, int bucket, int variant, int jt,
                                           int nsplit);
/* Admit a system (HOST double[n][3] x, v; float m[n]); NBGB_ERR_NO_MEMORY if
   no slot or arena space is free.  Its first tick computes its initial
   accelerations; each later tick is one KDK step of size dt, `steps` times. */
NBGB_API int nbgb_ensemble_add(nbgb_ensemble *ens, const double *pos3, const double *vel3,
                               const float *mass, size_t n, double dt, long long steps,
                               int *slot);
NBGB_API int nbgb_ensemble_tick(nbgb_ensemble *ens, int nticks);
NBGB_API int nbgb_ensemble_set_graph(nbgb_ensemble *ens, int enable);
NBGB_API int nbgb_ensemble_synchronize(nbgb_ensemble *ens);
/* Up to max slots whose steps are done; returns the count. */
NBGB_API int nbgb_ensemble_finished(nbgb_ensemble *ens, int *slots, int max);
/* HOST double[n][3] x, v and float4 accelerations (any may be NULL). */
NBGB_API int nbgb_ensemble_get_state(nbgb_ensemble *ens, int slot, double *pos3, double *vel3,
                                     float *acc4);
/* info[6]: bodies, steps done, steps left, variant, tile, j-split. */
NBGB_API int nbgb_ensemble_slot_info(nbgb_ensemble *ens, int slot, long long *info6);
/* Steps a system takes per tick, 1..8 (default 1), from the next tick on: a
   tick runs up to 8 passes, pass p moving the systems whose sub exceeds p, so
   small systems advance several steps while large ones advance one.  Each
   step is the same KDK step of size dt, so results do not depend on sub.  A
   system with s steps then finishes after 1 + ceil(s / sub) ticks. */
NBGB_API int nbgb_ensemble_set_substeps(nbgb_ensemble *ens, int slot, int sub);
/* CTAs of the persistent force launch, 1..nbgb_ensemble_max_grid (SMs x
   resident CTAs per SM; 0 = all, the default).  Two ensembles whose grids
   together fit the resident slots run side by side on their own streams. */
NBGB_API int nbgb_ensemble_set_grid(nbgb_ensemble *ens, int ctas);
NBGB_API int nbgb_ensemble_max_grid(nbgb_ensemble *ens);
/* Systems admitted afterwards with N >= nmin are evaluated with the
   Newton's-third-law kernel (as nbgb_force_newton3: each pair once, FP64
   block-pair sums) instead of the work queue; 0 = none (the default).  Their
   results repeat to FP64 rounding order rather than bit for bit.  The first
   nonzero call allocates an FP64 sums arena (24 B per body of capacity). */
NBGB_API int nbgb_ensemble_set_newton3_min(nbgb_ensemble *ens, size_t nmin);
/* high != 0: the ensemble's stream gets the device's greatest priority, so
   its CTAs are dispatched ahead of other streams' pending ones (an ensemble
   running beside a busier one).  Drains and recreates the stream. */
NBGB_API int nbgb_ensemble_set_priority(nbgb_ensemble *ens, int high);
NBGB_API int nbgb_ensemble_remove(nbgb_ensemble *ens, int slot);
NBGB_API int nbgb_ensemble_active(nbgb_ensemble *ens);
NBGB_API void *nbgb_ensemble_stream(nbgb_ensemble *ens);

/* ======================================================================== */
/* Initial conditions and error statistics (host)                            */
/* ======================================================================== */

/* Replaces: seedRandom + randomUnitBodies (src/nbody_util.cpp:81-144) as the
   driver calls them (src/nbody.cu:919, 996; scale 0.9, velscale 8): same LCG,
   same rejection order, so equal seeds give equal bodies.  HOST float4. */
NBGB_API int nbgb_ic_reference(float *posMass, float *velInvMass, size_t N, float scale,
                               float velscale, unsigned seed);
/* Uniform ball of the given radius, masses U[m_lo, m_hi] / N, zero
   velocities (velInvMass may be NULL).  HOST float4. */
NBGB_API int nbgb_ic_uniform_ball(float *posMass, float *velInvMass, size_t N, double radius,
                                  double m_lo, double m_hi, unsigned long long seed);
/* Plummer sphere (G = M = a = 1, equal masses, virial velocities).  Any of
   the FP64 double[N][3] or FP32 float4 outputs may be NULL. */
NBGB_API int nbgb_ic_plummer(double *pos3, double *vel3, float *posMass, float *velInvMass,
                             size_t N, unsigned long long seed);

/* Replaces: the crosscheck loop (src/nbody.cu:120-125, 406-418): max over
   bodies and x,y,z of |a - b| / b (signed b).  HOST float4. */
NBGB_API float nbgb_crosscheck_max_rel_error(const float *force, const float *golden, size_t N);
/* FP64 all-pairs force (double[n_targets][3]) and potential (self pair
   excluded; phi may be NULL) of the listed targets of a HOST float4 posMass,
   on the host's threads: the library's FP64 yardstick for its FP32 results.
   Pass eps2 as the binary32 value the GPU used. */
NBGB_API int nbgb_force_f64_host(const float *posMass, size_t N, double eps2,
                                 const long long *idx, size_t n_targets, double *force3,
                                 double *phi);
/* Per-body |F - T| / |T| against FP64 truth double[n_rows][3]; row t is body
   idx[t] (idx NULL: body t).  Max and RMS over rows. */
NBGB_API int nbgb_force_error_stats(const float *force, const double *truth3,
                                    const long long *idx, size_t n_rows, double *max_rel,
                                    double *rms_rel);

/* ======================================================================== */
/* Pipe-throughput microbenchmarks (roofline denominators)                   */
/* ======================================================================== */

/* which: 0 = scalar FP32 FMA (FLOP/s, FMA = 2), 1 = packed f32x2 FMA
   (FLOP/s), 2 = MUFU rsqrt (results/s), 3 = packed add, 4 = packed multiply
   (FLOP/s, 2 per instruction), 5 = packed FMA with three varying register
   operands, 6 = packed FMA with one MUFU rsqrt per six (FLOP/s of the
   FMAs), 7 = packed and scalar FMA interleaved, 8 = the force kernel's
   pair interaction on register-resident sources (20 FLOP/interaction),
   9 / 10 = MUFU ex2 / lg2, 11..16 = the pair interaction with some source
   pairs in the log-domain form, 17 = FP64 FMA (FLOP/s).  Full-GPU launch of `iters` x 128 operations per
   thread, best of `reps` after a warm-up.  Synchronous. */
NBGB_API int nbgb_measure_peak(int which, int iters, int reps, double *rate, float *ms);

/* One streaming copy kernel moving `bytes` (half read, half written) with L2
   evicted before each of `reps` launches: median GB/s and ms.  The measured
   cost of a short HBM-bound kernel on this GPU.  Synchronous. */
NBGB_API int nbgb_measure_copy(size_t bytes, int reps, double *gb_per_s, float *ms);

/* ======================================================================== */
/* Status                                                                    */
/* ======================================================================== */

/* Reads and clears the device status word of the current device (bits
   NBGB_STATUS_*).  Returns the bits, or a negative NBGB_ERR_* code. */
NBGB_API int nbgb_last_status(void);
NBGB_API const char *nbgb_status_string(int code);
/* Self-test of the bounded waits: a kernel waits on an mbarrier that nothing
   completes, gives up after limit_ms (0 < limit_ms <= 1000) and returns;
   returns the status bits it left (NBGB_STATUS_WAIT_TIMEOUT expected). */
NBGB_API int nbgb_selftest_bounded_wait(double limit_ms);

/* Checks the library's integer-pipe binary32 <-> binary64 conversions (used
   by the FP64 integrate kernels) against the hardware conversions on n
   pseudo-random bit patterns of every class; *mismatches receives the number
   of differing results (0 expected).  No reference counterpart.
   Synchronous. */
NBGB_API int nbgb_selftest_conversions(long long n, unsigned long long seed,
                                       unsigned long long *mismatches);
/* Library / build identification. */
NBGB_API const char *nbgb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NBODY_GB300_H */
