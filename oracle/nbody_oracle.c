/*
 * nbody_oracle.c -- CPU FP64 restatement of AstroNbodySim.jl's direct-summation
 * gravity path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and
 * the CPU-baseline leg of the benchmark load it as the checker.  The product
 * (libnbody_gb300.so) never links, loads or calls this file.
 *
 * What it restates (paths inside the AstroNbodySim.jl project):
 *   - pair force, Gadget-2 cubic spline      src/directsum/gravity.jl:8-28
 *   - per-target force sum (all j, incl. j=i) src/directsum/gravity.jl:37-46
 *   - active-particle force loop             src/directsum/gravity.jl:80-101
 *   - pair potential per unit mass           src/directsum/potential.jl:2-27
 *   - per-target potential sum               src/directsum/potential.jl:33-41, 67-79
 *   - total potential  0.5*sum(pot.*m)       src/directsum/potential.jl:150-153, src/base/Energy.jl:53-61
 *   - timestep criterion + power-of-two bin  src/base/Timestep.jl:1-23
 *   - init / adaptive kick / const kick      src/base/Timestep.jl:29-93
 *   - leapfrog half kicks                    src/base/Timestep.jl:105-125
 *   - min end step, drift                    src/base/Timestep.jl:135-195
 *   - drift split at snapshot times          src/base/Timestep.jl:197-245 (find_next_sync_point_and_drift)
 *   - snapshot schedule                      src/base/Config.jl:436-439, 749-750
 *   - step = drift -> force -> kick          src/directsum/timestep.jl:43-55
 *   - run loop (force, init, half kick, steps, back half kick)  src/run.jl:76-87, 101-173
 *   - kinetic energy, momentum, angular mom. src/base/Energy.jl:13-101
 *
 * Julia's `sum` over a Vector is Base's blocked pairwise reduction (sequential
 * below 16 elements, recursive halving above a block of 1024).  `jl_sum*` below
 * restate that algorithm so the summation order follows the reference; the
 * "truth" mode instead uses Neumaier-compensated summation to separate
 * summation-order noise from real differences.
 *
 * Parity pinning: the reference (Julia) cannot run in this environment.  The
 * oracle is pinned against the closed-form known answers that the reference's
 * own tests use (test/StaticTest.jl binary and box cases, test/Local-Timestep.jl
 * hand integrators), restated in tests/golden/.
 *
 * Build: -O2 -fno-fast-math -ffp-contract=off (Julia does not contract a*b+c
 * into an FMA unless asked), OpenMP static blocks over targets like split_block.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_LAW_SPLINE_G2 0
#define OR_LAW_PLUMMER 1

#define OR_CRIT_REF 0          /* dt = sqrt(2 eta h / |a|)   src/base/Timestep.jl:3 */
#define OR_CRIT_ETA_SQRT_EPS 1 /* dt = eta sqrt(h / |a|)     (alternative criterion) */

#define OR_OK 0
#define OR_ERR_MINSTEP -10
#define OR_ERR_TISTEP -11
#define OR_ERR_ARG -1

/* ------------------------------------------------------------------------- */
/* Julia Base pairwise sum (Base._mapreduce / Base.mapreduce_impl)            */
/* ------------------------------------------------------------------------- */
static double jl_sum_impl(const double *a, int64_t lo, int64_t hi)
{
    /* hi inclusive */
    if (lo == hi) return a[lo];
    if (hi - lo < 1024) {
        double v = a[lo] + a[lo + 1];
        for (int64_t i = lo + 2; i <= hi; ++i) v = v + a[i];
        return v;
    }
    int64_t mid = lo + ((hi - lo) >> 1);
    double v1 = jl_sum_impl(a, lo, mid);
    double v2 = jl_sum_impl(a, mid + 1, hi);
    return v1 + v2;
}

double or_jl_sum(const double *a, int64_t n)
{
    if (n <= 0) return 0.0;
    if (n == 1) return a[0];
    if (n < 16) {
        double s = a[0] + a[1];
        for (int64_t i = 2; i < n; ++i) s = s + a[i];
        return s;
    }
    return jl_sum_impl(a, 0, n - 1);
}

/* Neumaier compensated sum ("truth" mode). */
double or_compensated_sum(const double *a, int64_t n)
{
    double s = 0.0, c = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double t = s + a[i];
        if (fabs(s) >= fabs(a[i])) c += (s - t) + a[i];
        else c += (a[i] - t) + s;
        s = t;
    }
    return s + c;
}

static double sum_mode(const double *a, int64_t n, int mode)
{
    return mode == 0 ? or_jl_sum(a, n) : or_compensated_sum(a, n);
}

/* ------------------------------------------------------------------------- */
/* Pair kernels                                                              */
/* ------------------------------------------------------------------------- */

/* src/directsum/gravity.jl:8-28  (law SPLINE_G2); PLUMMER is the r^2+h^2 form
 * of the commented variant at src/directsum/gravity.jl:2-6.  Evaluation order
 * follows Julia's left-to-right evaluation of each expression. */
static inline void pair_force(double px, double py, double pz, double sx, double sy, double sz,
                              double m, double G, double h, int law, double *fx, double *fy,
                              double *fz)
{
    double dx = sx - px, dy = sy - py, dz = sz - pz;
    double r2 = dx * dx + dy * dy + dz * dz;
    double fac;
    if (law == OR_LAW_PLUMMER) {
        double r2e = r2 + h * h;
        fac = m / (r2e * sqrt(r2e));
    } else {
        double r = sqrt(r2);
        double h_inv = 1.0 / h;
        double h3_inv = h_inv * h_inv * h_inv;
        if (r >= h) {
            fac = m / (r2 * r);
        } else {
            double u = r * h_inv;
            if (u < 0.5) {
                fac = m * h3_inv * (10.666666666667 + u * u * (32.0 * u - 38.4));
            } else {
                fac = m * h3_inv *
                      (21.333333333333 - 48.0 * u + 38.4 * (u * u) - 10.666666666667 * (u * u * u) -
                       0.066666666667 / (u * u * u));
            }
        }
    }
    *fx = dx * fac * G;
    *fy = dy * fac * G;
    *fz = dz * fac * G;
}

/* src/directsum/potential.jl:2-27 */
static inline double pair_potential(double px, double py, double pz, double sx, double sy,
                                    double sz, double m, double G, double h, int law)
{
    double dx = sx - px, dy = sy - py, dz = sz - pz;
    double r2 = dx * dx + dy * dy + dz * dz;
    double r = sqrt(r2);
    double pot;
    if (law == OR_LAW_PLUMMER) {
        pot = -m / sqrt(r2 + h * h) * G;
    } else {
        double h_inv = 1.0 / h;
        if (r >= h) {
            pot = -m / r * G;
        } else {
            double u = r * h_inv;
            double wp;
            if (u < 0.5)
                wp = -2.8 + u * u * (5.333333333333 + u * u * (6.4 * u - 9.6));
            else
                wp = -3.2 + 0.066666666667 / u +
                     u * u * (10.666666666667 + u * (-16.0 + u * (9.6 - 2.133333333333 * u)));
            pot = m * h_inv * wp * G;
        }
    }
    if (r == 0.0) pot = pot * 0.0;
    return pot;
}

/* ------------------------------------------------------------------------- */
/* Force / potential at targets                                              */
/* ------------------------------------------------------------------------- */

/*
 * For every target t with active[t] != 0 (or all if active == NULL):
 *   acc[t] = sum_j pair_force(target t, source j, h[t])   (gravity.jl:37-46, 96-98)
 *   pot[t] = sum_j pair_potential(...)                    (potential.jl:33-41, 77)
 * mode 0: Julia pairwise sum order; mode 1: compensated ("truth").
 * Inactive targets keep whatever their output slots held (gravity.jl:96-99).
 */
int or_force(int64_t n_src, const double *sx, const double *sy, const double *sz, const double *sm,
             int64_t n_tgt, const double *tx, const double *ty, const double *tz, const double *th,
             const uint8_t *active, double G, int law, int mode, double *ax, double *ay,
             double *az, double *pot, int nthreads)
{
    if (n_src < 0 || n_tgt < 0) return OR_ERR_ARG;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int err = 0;
#pragma omp parallel
    {
        double *bx = (double *)malloc(sizeof(double) * (size_t)(n_src > 0 ? n_src : 1));
        double *by = (double *)malloc(sizeof(double) * (size_t)(n_src > 0 ? n_src : 1));
        double *bz = (double *)malloc(sizeof(double) * (size_t)(n_src > 0 ? n_src : 1));
        if (!bx || !by || !bz) {
#pragma omp atomic write
            err = 1;
        } else {
#pragma omp for schedule(static)
            for (int64_t t = 0; t < n_tgt; ++t) {
                if (active && !active[t]) continue;
                double px = tx[t], py = ty[t], pz = tz[t], h = th[t];
                if (ax) {
                    for (int64_t j = 0; j < n_src; ++j)
                        pair_force(px, py, pz, sx[j], sy[j], sz[j], sm[j], G, h, law, &bx[j], &by[j],
                                   &bz[j]);
                    ax[t] = sum_mode(bx, n_src, mode);
                    ay[t] = sum_mode(by, n_src, mode);
                    az[t] = sum_mode(bz, n_src, mode);
                }
                if (pot) {
                    for (int64_t j = 0; j < n_src; ++j)
                        bx[j] = pair_potential(px, py, pz, sx[j], sy[j], sz[j], sm[j], G, h, law);
                    pot[t] = sum_mode(bx, n_src, mode);
                }
            }
        }
        free(bx);
        free(by);
        free(bz);
    }
    return err ? OR_ERR_ARG : OR_OK;
}

/* ------------------------------------------------------------------------- */
/* Integrator state (structure-of-arrays, FP64, Int64 timeline)              */
/* ------------------------------------------------------------------------- */

typedef struct or_state {
    int64_t n;
    double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *pot, *m;
    int32_t *type; /* 1..6, index into softening table (Config.jl:108) */
    int64_t *ti_beg, *ti_end;
    double soft[6];
    double G;
    int32_t law;
    int32_t adaptive; /* 0: ConstantTimestep, 1: AdaptiveTimestep */
    int32_t criterion;
    int32_t nthreads;
    double dt;         /* ConstantTimestep.dt */
    double eta;        /* ErrTolTimestep */
    double min_step, max_step;
    int64_t time_base; /* TimeBase (1<<30) */
    double time_interval;
    /* TimeInfo */
    int64_t t_int, last_t_int;
    double t_float, last_t_float;
    int32_t mode; /* summation mode for forces */
    int32_t pad;
    /* force post-processing (src/base/PostProcessing/Force.jl:33-47) */
    int32_t bg_kind; /* 0 none, 1 point mass, 2 pseudo-Newtonian */
    int32_t mond;    /* 0 Newton, 1 Milgrom (1983) */
    double bg_gm, bg_cx, bg_cy, bg_cz, bg_rg;
    double mond_acc0, mond_nu_index;
    /* TimeConfig.Begin and the snapshot schedule: BetweenSnapshots,
     * BetweenSnapshotsInt = floor(BetweenSnapshots / TimeInterval) (adaptive)
     * (src/base/Config.jl:436-439) and TimeInfo.next_output_time_int/_float,
     * starting at BetweenSnapshotsInt / Begin + BetweenSnapshots
     * (src/base/Config.jl:749-750). outputs_on 0: no snapshots. */
    double time_begin;
    int32_t outputs_on;
    int32_t pad2;
    double between_float;
    int64_t between_int;
    double next_out_float;
    int64_t next_out_int;
    /* Snapshot sink (what sim.config.output.func sees): record k holds
     * t_float, t_int, then x, y, z, vx, vy, vz (n each); snap_count counts
     * every output, records beyond snap_cap are not stored. */
    double *snap;
    int64_t snap_cap, snap_count;
} or_state;

static inline double soft_of(const or_state *s, int64_t i) { return s->soft[s->type[i] - 1]; }

/* src/base/Timestep.jl:1-23 */
static int get_timestep(const or_state *s, double ax, double ay, double az, double h,
                        int64_t *out)
{
    double ac = sqrt(ax * ax + ay * ay + az * az);
    double dt;
    if (s->criterion == OR_CRIT_ETA_SQRT_EPS)
        dt = s->eta * sqrt(h / ac);
    else
        dt = sqrt(2 * s->eta * h / ac);
    if (dt > s->max_step) dt = s->max_step;
    if (dt < s->min_step) return OR_ERR_MINSTEP;
    double ti_step = dt / s->time_interval;
    if (!(ti_step > 0)) return OR_ERR_TISTEP;
    int64_t ti_min = s->time_base;
    while ((double)ti_min > ti_step) ti_min >>= 1;
    *out = ti_min;
    return OR_OK;
}

/* postprocessing_force for the CPU (src/base/PostProcessing/Force.jl:33-47):
 * background field of the active particles (bgforce closures; the point-mass
 * attractor of test/Local-Timestep.jl:746, the pseudo-Newtonian field of
 * src/tools/BlackHole.jl:41-60), then Milgrom (1983) MOND
 * (src/mond/milgrom1983.jl:6-8, 36-51).  a = 0 stays 0 under MOND. */
static void postprocess(or_state *s, const uint8_t *act)
{
    if (s->bg_kind == 0 && s->mond == 0) return;
    for (int64_t i = 0; i < s->n; ++i) {
        if (!act[i]) continue;
        double a0 = s->ax[i], a1 = s->ay[i], a2 = s->az[i];
        if (s->bg_kind != 0) {
            double rx = s->x[i] - s->bg_cx, ry = s->y[i] - s->bg_cy, rz = s->z[i] - s->bg_cz;
            double r2 = rx * rx + ry * ry + rz * rz;
            double r = sqrt(r2);
            double f;
            if (s->bg_kind == 1) {
                f = -s->bg_gm / r2;
            } else {
                double d = r - s->bg_rg;
                f = -s->bg_gm / (d * d);
            }
            a0 = a0 + f * (rx / r);
            a1 = a1 + f * (ry / r);
            a2 = a2 + f * (rz / r);
        }
        if (s->mond == 1) {
            double an = sqrt(a0 * a0 + a1 * a1 + a2 * a2);
            if (an > 0.0) {
                double y = an / s->mond_acc0;
                double nu = pow(0.5 * (1.0 + sqrt(1.0 + 4.0 * pow(y, -s->mond_nu_index))),
                                1.0 / s->mond_nu_index);
                a0 = a0 * nu;
                a1 = a1 * nu;
                a2 = a2 * nu;
            }
        }
        s->ax[i] = a0;
        s->ay[i] = a1;
        s->az[i] = a2;
    }
}

/* Force on active particles: gravity.jl:80-101 (active = Ti_endstep == now),
 * then the post-processing above. */
int or_compute_force(or_state *s, int want_pot)
{
    int64_t n = s->n;
    double *th = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    uint8_t *act = (uint8_t *)malloc((size_t)(n > 0 ? n : 1));
    if (!th || !act) {
        free(th);
        free(act);
        return OR_ERR_ARG;
    }
    for (int64_t i = 0; i < n; ++i) {
        th[i] = soft_of(s, i);
        act[i] = (uint8_t)(s->ti_end[i] == s->t_int);
    }
    int rc = or_force(n, s->x, s->y, s->z, s->m, n, s->x, s->y, s->z, th, act, s->G, s->law,
                      s->mode, s->ax, s->ay, s->az, want_pot ? s->pot : NULL, s->nthreads);
    if (rc == OR_OK) postprocess(s, act);
    free(th);
    free(act);
    return rc;
}

/* Potential of all particles: potential.jl:67-79 (every particle, softening of its type). */
int or_compute_potential(or_state *s)
{
    int64_t n = s->n;
    double *th = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (!th) return OR_ERR_ARG;
    for (int64_t i = 0; i < n; ++i) th[i] = soft_of(s, i);
    int rc = or_force(n, s->x, s->y, s->z, s->m, n, s->x, s->y, s->z, th, NULL, s->G, s->law,
                      s->mode, NULL, NULL, NULL, s->pot, s->nthreads);
    free(th);
    return rc;
}

/* src/base/Timestep.jl:29-39 */
int or_init_timesteps(or_state *s)
{
    for (int64_t i = 0; i < s->n; ++i) {
        if (!s->adaptive) {
            s->ti_end[i] = 0;
            continue;
        }
        int64_t b;
        int rc = get_timestep(s, s->ax[i], s->ay[i], s->az[i], soft_of(s, i), &b);
        if (rc) return rc;
        s->ti_end[i] = b;
    }
    return OR_OK;
}

/* src/base/Timestep.jl:105-125 */
int or_half_kick(or_state *s, int forward)
{
    double fw = (double)forward;
    for (int64_t i = 0; i < s->n; ++i) {
        if (s->adaptive) {
            double d = (double)(s->ti_end[i] - s->ti_beg[i]);
            s->vx[i] = s->vx[i] + s->ax[i] * fw * 0.5 * d * s->time_interval;
            s->vy[i] = s->vy[i] + s->ay[i] * fw * 0.5 * d * s->time_interval;
            s->vz[i] = s->vz[i] + s->az[i] * fw * 0.5 * d * s->time_interval;
        } else {
            s->vx[i] = s->vx[i] + s->ax[i] * fw * 0.5 * s->dt;
            s->vy[i] = s->vy[i] + s->ay[i] * fw * 0.5 * s->dt;
            s->vz[i] = s->vz[i] + s->az[i] * fw * 0.5 * s->dt;
        }
    }
    return OR_OK;
}

/* src/base/Timestep.jl:47-93 */
int or_kick(or_state *s)
{
    if (!s->adaptive) {
        for (int64_t i = 0; i < s->n; ++i) {
            s->vx[i] = s->vx[i] + s->ax[i] * s->dt;
            s->vy[i] = s->vy[i] + s->ay[i] * s->dt;
            s->vz[i] = s->vz[i] + s->az[i] * s->dt;
        }
        return OR_OK;
    }
    int64_t TB = s->time_base;
    for (int64_t i = 0; i < s->n; ++i) {
        if (s->ti_end[i] != s->t_int) continue;
        int64_t ti_step;
        int rc = get_timestep(s, s->ax[i], s->ay[i], s->az[i], soft_of(s, i), &ti_step);
        if (rc) return rc;
        if (s->t_int == TB) ti_step = 0;
        if (TB - s->t_int < ti_step) ti_step = TB - s->t_int;
        double tstart = (double)(s->ti_beg[i] + s->ti_end[i]) / 2;
        double tend = (double)s->ti_end[i] + 0.5 * (double)ti_step;
        double dt = (tend - tstart) * s->time_interval;
        s->vx[i] = s->vx[i] + s->ax[i] * dt;
        s->vy[i] = s->vy[i] + s->ay[i] * dt;
        s->vz[i] = s->vz[i] + s->az[i] * dt;
        s->ti_beg[i] = s->ti_end[i];
        s->ti_end[i] = s->ti_beg[i] + ti_step;
    }
    return OR_OK;
}

/* src/base/Timestep.jl:135-144 */
int64_t or_find_min_endstep(const or_state *s)
{
    int64_t mn = s->time_base;
    for (int64_t i = 0; i < s->n; ++i)
        if (mn > s->ti_end[i]) mn = s->ti_end[i];
    return mn;
}

static void drift_by(or_state *s, double dt)
{
    for (int64_t i = 0; i < s->n; ++i) {
        s->x[i] = s->x[i] + s->vx[i] * dt;
        s->y[i] = s->y[i] + s->vy[i] * dt;
        s->z[i] = s->z[i] + s->vz[i] * dt;
    }
}

/* Adaptive drift to an integer time: src/directsum/timestep.jl:1-20 + Timestep.jl:169-179 */
int or_drift_to_int(or_state *s, int64_t next_int)
{
    s->last_t_int = s->t_int;
    s->t_int = next_int;
    s->t_float = s->time_begin + (double)s->t_int * s->time_interval;
    double dt = (double)(s->t_int - s->last_t_int) * s->time_interval;
    drift_by(s, dt);
    return OR_OK;
}

/* Constant drift to a float time: src/directsum/timestep.jl:22-38 + Timestep.jl:181-191 */
int or_drift_to_float(or_state *s, double next_float)
{
    s->last_t_float = s->t_float;
    s->t_float = next_float;
    double dt = s->t_float - s->last_t_float;
    drift_by(s, dt);
    return OR_OK;
}

/* sim.config.output.func: one snapshot record of the current state. */
static void or_output(or_state *s)
{
    const int64_t n = s->n;
    if (s->snap && s->snap_count < s->snap_cap) {
        double *r = s->snap + s->snap_count * (2 + 6 * n);
        r[0] = s->t_float;
        r[1] = (double)s->t_int;
        memcpy(r + 2 + 0 * n, s->x, sizeof(double) * (size_t)n);
        memcpy(r + 2 + 1 * n, s->y, sizeof(double) * (size_t)n);
        memcpy(r + 2 + 2 * n, s->z, sizeof(double) * (size_t)n);
        memcpy(r + 2 + 3 * n, s->vx, sizeof(double) * (size_t)n);
        memcpy(r + 2 + 4 * n, s->vy, sizeof(double) * (size_t)n);
        memcpy(r + 2 + 5 * n, s->vz, sizeof(double) * (size_t)n);
    }
    s->snap_count += 1;
}

/* find_next_sync_point_and_drift: src/base/Timestep.jl:197-215 (constant:
 * drift to every output time up to t + dt, writing a snapshot at each, then
 * to t + dt) and :224-245 (adaptive: the same on the integer time line up to
 * min_endstep). */
int or_sync_and_drift(or_state *s)
{
    if (s->adaptive) {
        const int64_t mn = or_find_min_endstep(s);
        if (s->outputs_on && s->between_int <= 0) return OR_ERR_ARG;
        while (s->outputs_on && s->next_out_int <= mn) {
            or_drift_to_int(s, s->next_out_int);
            or_output(s);
            s->next_out_int += s->between_int;
        }
        return or_drift_to_int(s, mn);
    }
    const double next_system_time = s->t_float + s->dt;
    if (s->outputs_on && !(s->between_float > 0.0)) return OR_ERR_ARG;
    while (s->outputs_on && s->next_out_float <= next_system_time) {
        or_drift_to_float(s, s->next_out_float);
        or_output(s);
        s->next_out_float += s->between_float;
    }
    return or_drift_to_float(s, next_system_time);
}

/* One step, src/directsum/timestep.jl:43-55: find_next_sync_point_and_drift,
 * force on the active particles, kick. */
int or_step(or_state *s)
{
    int rc = or_sync_and_drift(s);
    if (rc) return rc;
    rc = or_compute_force(s, 0);
    if (rc) return rc;
    rc = or_kick(s);
    if (!s->adaptive) s->last_t_float = s->t_float; /* run.jl:164 */
    return rc;
}

/* src/run.jl:76-87 (warm-up force, init timesteps, forward half kick). */
int or_run_begin(or_state *s)
{
    int rc = or_compute_force(s, 0);
    if (rc) return rc;
    rc = or_init_timesteps(s);
    if (rc) return rc;
    return or_half_kick(s, +1);
}

/* src/run.jl:171-173 */
int or_run_end(or_state *s) { return or_half_kick(s, -1); }

/* ------------------------------------------------------------------------- */
/* Diagnostics: src/base/Energy.jl                                           */
/* ------------------------------------------------------------------------- */

/* out[0]=K, out[1]=W (0.5*sum(pot.*m), needs s->pot), out[2..4]=P, out[5..7]=L */
int or_diagnostics(const or_state *s, double *out)
{
    int64_t n = s->n;
    double *b = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (!b) return OR_ERR_ARG;
    for (int64_t i = 0; i < n; ++i) {
        double hm = 0.5 * s->m[i];
        b[i] = (hm * s->vx[i]) * s->vx[i] + (hm * s->vy[i]) * s->vy[i] + (hm * s->vz[i]) * s->vz[i];
    }
    out[0] = or_jl_sum(b, n);
    for (int64_t i = 0; i < n; ++i) b[i] = s->pot[i] * s->m[i];
    out[1] = 0.5 * or_jl_sum(b, n);
    for (int64_t i = 0; i < n; ++i) b[i] = s->vx[i] * s->m[i];
    out[2] = or_jl_sum(b, n);
    for (int64_t i = 0; i < n; ++i) b[i] = s->vy[i] * s->m[i];
    out[3] = or_jl_sum(b, n);
    for (int64_t i = 0; i < n; ++i) b[i] = s->vz[i] * s->m[i];
    out[4] = or_jl_sum(b, n);
    for (int64_t i = 0; i < n; ++i) b[i] = s->m[i] * (s->y[i] * s->vz[i] - s->z[i] * s->vy[i]);
    out[5] = or_jl_sum(b, n);
    for (int64_t i = 0; i < n; ++i) b[i] = s->m[i] * (s->z[i] * s->vx[i] - s->x[i] * s->vz[i]);
    out[6] = or_jl_sum(b, n);
    for (int64_t i = 0; i < n; ++i) b[i] = s->m[i] * (s->x[i] * s->vy[i] - s->y[i] * s->vx[i]);
    out[7] = or_jl_sum(b, n);
    free(b);
    return OR_OK;
}

int or_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
