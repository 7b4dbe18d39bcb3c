/*
 * nbody_gb300.h -- C ABI of libnbody_gb300.so, the GB300 (sm_103a) direct-sum
 * gravity engine that stands in for AstroNbodySim.jl's DirectSum GPU device.
 *
 * Every entry point is plain C (pointers, sizes, status codes).  The library
 * owns all device memory behind an opaque handle; host arrays are read only
 * during an upload call and written only during a download call.  One CUDA
 * stream per handle; calls on one handle must be serialised by the caller,
 * distinct handles may be driven from different threads.
 *
 * Reference interfaces each entry point replaces are cited as
 * path:line inside the AstroNbodySim.jl project.
 */
#ifndef NBODY_GB300_H
#define NBODY_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (0 = success) -------------------------------------- */
#define NB_OK 0
#define NB_ERR_INVALID_ARG -1
#define NB_ERR_OOM -2
#define NB_ERR_CUDA -3
#define NB_ERR_NUMERIC -4  /* NaN/Inf acceleration, dt < MinStep, bad integer step
                              (src/base/Timestep.jl:9-16) */
#define NB_ERR_TIMEOUT -5  /* a bounded device-side wait gave up */
#define NB_ERR_ADMISSION -6 /* batch/serve: request does not fit the footprint budget */
#define NB_ERR_STATE -7    /* call out of order (e.g. no particles uploaded) */
#define NB_ERR_NOT_FOUND -8 /* batch/serve: unknown request id */

/* ---- enums ----------------------------------------------------------- */
#define NB_LAW_SPLINE_G2 0 /* Gadget-2 cubic spline, src/directsum/gravity.jl:8-28 */
#define NB_LAW_PLUMMER 1   /* a = G m d / (r^2 + h^2)^(3/2) */

#define NB_PREC_FP64 0  /* plain FP64 pair arithmetic, the reference's Float64 form */
#define NB_PREC_MIXED 1 /* FP32 pairs relative to FP64 tile origins, compensated sums */

#define NB_CRIT_REF 0          /* dt = sqrt(2 eta h / |a|), src/base/Timestep.jl:3 */
#define NB_CRIT_ETA_SQRT_EPS 1 /* dt = eta sqrt(h / |a|) */

/* TimeIntegrationAlgorithm (src/base/Config.jl:398, src/run.jl:85-87, 171-173) */
#define NB_ALG_LEAPFROG 0 /* run begins with a +1/2 kick and ends with a -1/2 kick */
#define NB_ALG_EULER 1    /* the same step loop without the half kicks */

/* flags of nb_compute_force */
#define NB_FORCE_POT 1 /* also write the potential per unit mass */

typedef struct nb_handle nb_handle;

/* Mirrors the SimConfig keywords relevant to DirectSum on GPU
 * (src/base/Config.jl:515-628, TimeConfig :408-449, GravityConfig :106-169). */
typedef struct nb_params {
    double G;             /* sim.config.constants.G (units stripped by the caller) */
    double softening[6];  /* ForceSofteningTable, indexed by particle type 1..6 */
    int32_t law;          /* NB_LAW_* */
    int32_t precision;    /* NB_PREC_* */
    int32_t adaptive;     /* 0: ConstantTimestep(dt); 1: AdaptiveTimestep */
    int32_t criterion;    /* NB_CRIT_* (adaptive only) */
    double dt;            /* TimeStep (constant) */
    double eta;           /* ErrTolTimestep (default 0.025) */
    double min_step;      /* MinStep (default 1e-8) */
    double max_step;      /* MaxStep (default +Inf) */
    int64_t time_base;    /* TimeBase (default 1<<30) */
    double time_begin;    /* TimeBegin */
    double time_end;      /* TimeEnd; TimeInterval = (end-begin)/time_base */
    int32_t device;       /* CUDA ordinal */
    int32_t tile_j;       /* tuning override: sources per j-tile, 128, 256 or 512 (0: 256 with an
                             explicit launch shape; with the built-in rule 128 below 2^15
                             particles, 256 below 2^17, 512 from there) */
    int32_t i_per_thread; /* tuning override (0 = auto) */
    int32_t block;        /* tuning override: threads per CTA of the direct grid (128, 256);
                             -1 = persistent work-list kernel; 0 (with i_per_thread 0) = auto */
    int32_t j_split;      /* tuning override: CTAs sharing one i-block's sources in the direct
                             grid (1..8; 0 = 1) */
    int32_t algorithm;    /* NB_ALG_LEAPFROG (default) or NB_ALG_EULER: whether nb_run_begin /
                             nb_run_end apply the half kicks; kept in checkpoint images */
    /* Force post-processing, applied by nb_compute_force and nb_step to the
     * particles that received a force (postprocessing_force,
     * src/directsumgpu/gravity.jl:64-79; CPU src/base/PostProcessing/Force.jl:33-47):
     * first an analytic background field (the reference's bgforce closures,
     * as the point-mass attractor of test/Local-Timestep.jl:746 or the
     * pseudo-Newtonian field of src/tools/BlackHole.jl:41-60), then the
     * Milgrom (1983) MOND correction a *= nu(|a| / ACC0, MOND_nuIndex)
     * (src/mond/milgrom1983.jl:6-8, 36-51). */
    int32_t bg_kind;      /* NB_BG_NONE, NB_BG_POINT_MASS, NB_BG_PSEUDO_NEWTONIAN */
    int32_t mond;         /* NB_MOND_NONE, NB_MOND_MILGROM1983 */
    double bg_gm;         /* G * M of the central object */
    double bg_center[3];  /* its position */
    double bg_rg;         /* gravity radius r_g of NB_BG_PSEUDO_NEWTONIAN */
    double mond_acc0;     /* ACC0 (> 0 when mond is set) */
    double mond_nu_index; /* MOND_nuIndex (reference default 2) */
    int32_t stages;       /* tuning override: depth of the force kernel's shared-memory ring of
                             j-tiles, 3, 4 or 6 (0 = 4) */
    int32_t resort_every; /* steps of nb_step / nb_step_until_output between Morton re-orders of
                             the sources (0 = 16; 1 = every step).  Steps in between pack the
                             sources in the last order, which stays a valid permutation: the
                             forces differ only by FP32 round-off.  Every other force call,
                             nb_upload and nb_checkpoint_load re-order first. */
} nb_params;

#define NB_BG_NONE 0
#define NB_BG_POINT_MASS 1
#define NB_BG_PSEUDO_NEWTONIAN 2
#define NB_MOND_NONE 0
#define NB_MOND_MILGROM1983 1

/* Energy / momentum diagnostics, FP64 (src/base/Energy.jl:13-101). */
typedef struct nb_diag {
    double kinetic;   /* sum 0.5 m v.v */
    double potential; /* 0.5 sum m phi (src/directsum/potential.jl:150-153) */
    double momentum[3];
    double angular_momentum[3];
} nb_diag;

/* Fill *p with the reference defaults (G=1, softening 1e-4, spline, mixed,
 * adaptive, eta 0.025, MinStep 1e-8, MaxStep Inf, TimeBase 2^30, [0, 0.1]). */
void nb_default_params(nb_params *p);

/* Create a handle on p->device.  Replaces the GPU branch of the Simulation
 * constructor's data placement (src/base/Config.jl:1072-1088). */
int nb_create(const nb_params *p, nb_handle **out);
int nb_destroy(nb_handle *h);

/* Use the caller's CUDA stream (a cudaStream_t passed as void*) instead of the
 * handle's own; NULL restores the handle's own stream. */
int nb_set_stream(nb_handle *h, void *stream);
int nb_get_stream(nb_handle *h, void **stream);

/* Upload n particles, SoA FP64; type[i] in 1..6 (Collection index into the
 * softening table, src/base/Config.jl:108).  Resets the time line (t_int = 0,
 * t_float = time_begin), Ti_begstep = Ti_endstep = 0, Acc = 0.
 * Replaces cu(StructArray(d)) at src/base/Config.jl:1072-1088. */
int nb_upload(nb_handle *h, int64_t n, const double *x, const double *y, const double *z,
              const double *vx, const double *vy, const double *vz, const double *m,
              const int32_t *type);

/* Download state; any pointer may be NULL.  Replaces get_all_data / get_local_data
 * (src/base/Config.jl:1199-1201, 1228-1230). */
int nb_download(nb_handle *h, double *x, double *y, double *z, double *vx, double *vy,
                double *vz, double *ax, double *ay, double *az, double *pot,
                int64_t *ti_begstep, int64_t *ti_endstep);

/* Overwrite accelerations / integer time bins (restart, tests). */
int nb_upload_acc(nb_handle *h, const double *ax, const double *ay, const double *az);
int nb_upload_bins(nb_handle *h, const int64_t *ti_begstep, const int64_t *ti_endstep);

/* Replaces set_softlen! for GPU (src/tools/SofteningLength.jl:87-89).
 * Every entry must be > 0 (h = 0 makes the reference's self pair 0/0). */
int nb_set_softening(nb_handle *h, const double soft[6]);

/* Acceleration of the active particles (Ti_endstep == system_time_int), all of
 * them in constant-step mode; inactive particles keep their Acc as on the CPU
 * path.  flags & NB_FORCE_POT also writes the potential of the same particles.
 * Replaces compute_force(sim, DirectSum, GPU) (src/directsumgpu/gravity.jl:36-45,
 * 81-85) with CPU semantics (src/directsum/gravity.jl:92-101). */
int nb_compute_force(nb_handle *h, int flags);

/* Potential per unit mass of every particle.  New GPU method for
 * compute_potential(sim, DirectSum, CPU) (src/directsum/potential.jl:142-148). */
int nb_compute_potential(nb_handle *h);

/* Self-potential term of src/base/Potential.jl:5-24: pot += G m / (h / 2.8)
 * for every particle (h from its type), as compute_potential(sim) applies it
 * after the direct sum (src/base/Potential.jl:21-24). */
int nb_remove_self_potential(nb_handle *h);

/* Acceleration and potential at n probe points (host arrays) with softening
 * length soft, from all resident particles.  Replaces
 * compute_force(sim, pos, SoftLength) (src/directsum/gravity.jl:180-193) and
 * compute_potential(sim, pos, SoftLength) (src/directsum/potential.jl:171-181).
 * Any output pointer may be NULL. */
int nb_force_at_points(nb_handle *h, int64_t n, const double *px, const double *py,
                       const double *pz, double soft, double *ax, double *ay, double *az,
                       double *pot);

/* init_timesteps (src/base/Timestep.jl:29-44; GPU src/directsumgpu/timestep.jl:32-47). */
int nb_init_timesteps(nb_handle *h);

/* leapfrog_half_kick with forward = +1 / -1 (src/base/Timestep.jl:105-133;
 * GPU src/directsumgpu/timestep.jl:178-214). */
int nb_half_kick(nb_handle *h, int forward);

/* advance_and_find_timestep (src/base/Timestep.jl:47-101; GPU :122-174). */
int nb_kick(nb_handle *h);

/* find_min_endstep (src/base/Timestep.jl:135-144; GPU src/directsumgpu/timestep.jl:103-114). */
int nb_find_min_endstep(nb_handle *h, int64_t *min_endstep);

/* drift_particles_adaptive_timestep to an integer time (src/directsum/timestep.jl:1-20)
 * and drift_particles_const_timestep to a float time (:22-38). */
int nb_drift_to_int(nb_handle *h, int64_t t_int);
int nb_drift_to_float(nb_handle *h, double t_float);

/* nsteps of step(sim, DirectSum, GPU) (src/directsumgpu/timestep.jl:216-224):
 * drift to the next sync point, force on active particles, kick.  The step is
 * captured once in a CUDA graph and replayed; the time line lives on the device. */
int nb_step(nb_handle *h, int64_t nsteps);

/* src/run.jl:76-87: force, init_timesteps, forward half kick (the half kick
 * only with NB_ALG_LEAPFROG). */
int nb_run_begin(nb_handle *h);

/* src/run.jl:171-173: the backward half kick with NB_ALG_LEAPFROG, nothing
 * with NB_ALG_EULER. */
int nb_run_end(nb_handle *h);

/* Snapshot schedule: TimeConfig.BetweenSnapshots (src/base/Config.jl:392-394,
 * 426, 436-439) and TimeInfo.next_output_time_int / _float
 * (src/base/Config.jl:749-750).  between > 0 sets the first output time to
 * TimeBegin + between (integer time line: BetweenSnapshotsInt =
 * floor(between / TimeInterval), which must be >= 1 with adaptive steps);
 * between = 0 turns output stops off (the default).  Call it before the run,
 * as the reference fixes the schedule when the Simulation is built; nb_upload
 * resets the schedule together with the time line.  With a schedule, every
 * step splits its drift at the output times inside it exactly as
 * find_next_sync_point_and_drift does (src/base/Timestep.jl:197-215 constant,
 * :224-245 adaptive): drift to the output time, output, next output time +=
 * BetweenSnapshots, then drift on to the step's end.  The reference's GPU
 * drift of constant steps always moves by the full dt
 * (src/directsumgpu/timestep.jl:67-74); this follows its CPU path. */
int nb_set_snapshot_interval(nb_handle *h, double between);

/* Up to max_steps steps of step(sim, DirectSum, GPU) that stop at the first
 * output time reached: then *at_output = 1, the positions are drifted to the
 * output time (velocities at the half step, as the reference's output
 * function sees them), nb_get_time gives the output time, and the caller
 * writes its snapshot (sim.config.output.func, src/base/Timestep.jl:204-206,
 * 234-236) before calling again, which finishes the interrupted step.
 * *steps_done counts completed steps.  Without a snapshot schedule this is
 * nb_step(h, max_steps).  nb_step itself, with a schedule, splits the drifts
 * the same way but does not stop. */
int nb_step_until_output(nb_handle *h, int64_t max_steps, int64_t *steps_done,
                         int32_t *at_output);

/* The snapshot schedule's state: next output time (integer and float; while
 * stopped at an output, the one after it), whether the time line is stopped
 * at an output, and the number of output stops so far.  Any pointer may be
 * NULL. */
int nb_get_output_time(nb_handle *h, int64_t *next_int, double *next_float, int32_t *at_output,
                       int64_t *outputs);

/* System time (TimeInfo.system_time_int / system_time_float). */
int nb_get_time(nb_handle *h, int64_t *t_int, double *t_float);

/* FP64 diagnostics; with_potential != 0 first recomputes the potential
 * (src/base/Energy.jl:13-101, src/directsum/potential.jl:150-153). */
int nb_diagnostics(nb_handle *h, int with_potential, nb_diag *out);

/* Steps taken by nb_step since the upload, and the pair evaluations they made
 * (active targets x all sources per step). */
int nb_get_counters(nb_handle *h, int64_t *steps, double *interactions);

/* check_sync_point for GPU (src/directsumgpu/timestep.jl:116-118,
 * src/base/Timestep.jl:146-157): *sync = 1 when every particle's Ti_endstep
 * is past the min_endstep of the last nb_find_min_endstep (or of the last
 * adaptive nb_step), i.e. the system is at a full synchronisation point. */
int nb_check_sync_point(nb_handle *h, int32_t *sync);

/* Number of particles active at the current time (Ti_endstep == t_int). */
int nb_active_count(nb_handle *h, int64_t *count);

/* Device-state checkpoint, replacing saverestart for (DirectSum, GPU)
 * (src/restart.jl:14-19) and loadrestart (src/restart.jl:129-139).  The image
 * is one host buffer: parameters, particles (x, v, a, pot, m, type,
 * Ti_begstep, Ti_endstep) and the device time line.  nb_checkpoint_size gives
 * its size for the current particle count; nb_checkpoint_save fills a buffer
 * of at least that size; nb_checkpoint_load replaces the state and parameters
 * of a handle (of any size, on its own device) with an image, after which the
 * run continues bit-identically to the saved one.  Images are checked for the
 * magic, version and sizes of this library and rejected with
 * NB_ERR_INVALID_ARG otherwise. */
int nb_checkpoint_size(nb_handle *h, int64_t *bytes);
int nb_checkpoint_save(nb_handle *h, void *buf, int64_t bytes);
int nb_checkpoint_load(nb_handle *h, const void *buf, int64_t bytes);

/* Mixed-precision acceleration (and, if pot != NULL, potential per unit mass)
 * of n particles from the same n particles, one softening length for all,
 * without allocating any device memory.  No counterpart in the reference: it
 * exists for callers that cannot let the library call cudaMalloc -- a Julia
 * host whose device arrays all come from CUDA.jl's pooled allocator, or a
 * serving process that reserves its HBM budget up front.  x, y, z, m, ax, ay,
 * az, pot are device pointers of the caller on the current device; stream is
 * a cudaStream_t (NULL = legacy default stream); the call synchronises the
 * stream before returning.  Scratch is one fixed device array of this library
 * (about 2.7 MB, held by every GPU that loads the library until exit), so
 * n must be 1..65536; larger n returns NB_ERR_INVALID_ARG with a message in
 * errbuf (may be NULL).  All calls share that array: calls that overlap on the
 * GPU race and must be serialised by the caller.  Every call reads an error
 * word back and synchronises its stream, so no call can run inside a stream
 * capture.
 * Results agree with nb_compute_force of a handle with NB_PREC_MIXED, the same
 * law, G and softening for every particle type, within the mixed-precision
 * tolerance: the same kernels, with another launch shape (128 threads x 2
 * targets, no j-split), so the FP32 sums run in another order. */
int nb_force_noalloc(int64_t n, const double *x, const double *y, const double *z,
                     const double *m, int32_t law, double G, double softening, double *ax,
                     double *ay, double *az, double *pot, void *stream, char *errbuf,
                     int64_t errbuf_len);

/* ---- many-system engine (batching and serving) -------------------------
 * No single counterpart in the reference: AstroNbodySim.jl runs one
 * Simulation at a time.  The engine keeps many independent systems resident in
 * one particle arena, advances all of them together with the same kernels as
 * step(sim, DirectSum, GPU) (constant-step leapfrog, mixed precision), and
 * admits queued systems as arena space and slots free up (continuous
 * batching).  Each system is integrated exactly as run(sim) does
 * (src/run.jl:76-87, 101-173): force, +1/2 kick, nsteps x (drift, force,
 * kick), -1/2 kick.  A system's result does not depend on the other systems in
 * the mix (bit-identical alone or together). */
typedef struct nb_engine nb_engine;

typedef struct nb_engine_params {
    double G;
    int32_t law;                /* NB_LAW_* for every system */
    int32_t device;
    int64_t max_particles;      /* arena capacity: the footprint budget of admission */
    int32_t max_systems;        /* resident system slots */
    int32_t max_steps_per_call; /* steps between admission rounds in nb_engine_run (0 = 64) */
    int32_t block;              /* tuning override: threads per CTA of the batch force (128, 256;
                                   0 = 128) */
    int32_t i_per_thread;       /* tuning override: targets per thread (1, 2; 0 = 2) */
} nb_engine_params;

#define NB_REQ_QUEUED 0
#define NB_REQ_RUNNING 1
#define NB_REQ_DONE 2
#define NB_REQ_CANCELLED 3
#define NB_REQ_SUSPENDED 4

typedef struct nb_engine_stats {
    int64_t queued;
    int64_t running;
    int64_t done;
    int64_t resident_particles;
    int64_t engine_steps;       /* engine steps executed (all resident systems advance) */
    double interactions;        /* sum over steps and systems of n^2 */
    double gpu_ms;              /* CUDA-event time of the engine steps */
} nb_engine_stats;

int nb_engine_create(const nb_engine_params *p, nb_engine **out);
int nb_engine_destroy(nb_engine *e);
/* Queue one system (host SoA arrays, copied): n particles, Plummer/spline
 * softening, constant dt, nsteps KDK steps.  Returns its id.  A system larger
 * than the whole arena or than a slot allows is rejected with NB_ERR_ADMISSION. */
int nb_batch_submit(nb_engine *e, int64_t n, const double *x, const double *y, const double *z,
                    const double *vx, const double *vy, const double *vz, const double *m,
                    double softening, double dt, int64_t nsteps, int64_t *id);
/* Admit what fits, then run a chunk of up to max_steps engine steps (at most
 * max_steps_per_call, and no more than the resident system with the most
 * steps left needs).  Every resident system advances one KDK step per engine
 * step until it has made its nsteps; a system that finishes inside the chunk
 * is held on the device where its last step left it (no drift, force or kick)
 * until the chunk ends.  *steps_done = engine steps of the chunk.  Finished
 * systems are then retired and their results kept for nb_batch_fetch. */
int nb_engine_run(nb_engine *e, int64_t max_steps, int64_t *steps_done);
/* The same as nb_engine_run, but the chunk of steps is only launched: the
 * call returns while the GPU works, so the caller can build and submit new
 * requests meanwhile (submit, poll, fetch and drain_done are host-side and do
 * not wait).  The next nb_engine_run / nb_engine_run_async / nb_engine_sync
 * (and cancel or suspend) first waits for the chunk, accounts it and retires
 * the systems it finished.  *steps_launched = steps of the chunk (0: nothing
 * was resident).  Statistics lag by the chunk in flight. */
int nb_engine_run_async(nb_engine *e, int64_t max_steps, int64_t *steps_launched);
/* Waits for the chunk left by nb_engine_run_async, if any. */
int nb_engine_sync(nb_engine *e);
int nb_batch_poll(nb_engine *e, int64_t id, int32_t *state, int64_t *steps_done);
/* Copy the final positions and velocities of a finished system (then forget it). */
int nb_batch_fetch(nb_engine *e, int64_t id, double *x, double *y, double *z, double *vx,
                   double *vy, double *vz);
int nb_batch_cancel(nb_engine *e, int64_t id);
/* Evict a running system to host memory (positions, half-step velocities,
 * accelerations, masses, its Morton order and step count), freeing its arena
 * range and slot; state NB_REQ_SUSPENDED.  nb_batch_resume queues it again
 * (FIFO); once re-admitted it continues without a new start-up force or half
 * kick, and its result is bit-identical to an uninterrupted run.  The
 * reference has no batch engine; this is the per-request form of its restart
 * files (src/restart.jl). */
int nb_batch_suspend(nb_engine *e, int64_t id);
int nb_batch_resume(nb_engine *e, int64_t id);
int nb_engine_get_stats(nb_engine *e, nb_engine_stats *out);
/* Ids of systems finished since the previous call (up to cap; *count set). */
int nb_engine_drain_done(nb_engine *e, int64_t *ids, int64_t cap, int64_t *count);
const char *nb_engine_last_error(nb_engine *e);

/* Self-test of the bounded-wait path (no counterpart in the reference): one
 * warp on `device` waits on an mbarrier that nothing completes, gives up after
 * timeout_ns (at most 2 s) exactly as the force kernels do on a copy that
 * never lands, records the timeout in a device error word and returns.
 * Returns NB_ERR_TIMEOUT (the expected outcome) with the time waited in
 * *waited_ms; the device context stays usable. */
int nb_selftest_wait_timeout(int device, int64_t timeout_ns, double *waited_ms);

/* FP32 throughput probe (no counterpart in the reference; it measures the
 * denominator of the force kernel's roofline): 4 CTAs x 256 threads per SM,
 * each thread running 8 independent chains of fma.rn.f32 (packed = 0) or
 * fma.rn.f32x2 (packed = 1, two lanes per instruction), timed with CUDA
 * events (best of 5 after a warm-up launch).  *tflops counts 2 flop per FMA
 * lane. */
int nb_selftest_fp32_peak(int device, int packed, double *tflops, double *ms);

/* Last error message of this handle (never NULL).  With a NULL handle: why the
 * last nb_create on the calling thread failed. */
const char *nb_last_error(nb_handle *h);

/* Library version string. */
const char *nb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NBODY_GB300_H */
