"""Generate the golden known-answer fixtures of tests/golden/*.json.

The reference (AstroNbodySim.jl) cannot run here, so its tests' known answers
are restated in plain Python from the closed forms and hand integrators that
the reference's own tests use:

  binary_static.json   test/StaticTest.jl:18-70, 161-207 (binary force, potential,
                       kinetic, energy, momentum, angular momentum, timestep bound),
                       unitless variant :210-297 with G = 1.
  box_probe.json       test/StaticTest.jl:92-123, 299-350 (force and potential of
                       the 10-particle box at the origin); the direct sum is
                       evaluated with math.fsum (correctly rounded sum of the pair
                       terms), independent of the oracle's summation order.
  circular_binary_const_leapfrog.json
                       test/Local-Timestep.jl:54-91, 219-247, 402-421 (hand
                       leapfrog of a circular binary, 2900 steps at
                       dt = sqrt(2 eta h / |a1|), final x and y).
  circular_binary_adaptive.json
                       src/base/Timestep.jl:1-82 and src/run.jl:76-173 restated
                       a second time in pure Python for a two-body system with
                       power-of-two bins (TimeBase 2^30), to pin the C oracle's
                       integer time line.

Run:  python tests/golden/make_golden.py   (writes next to this file)
"""
import json
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def w(name, obj):
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(obj, f, indent=1, sort_keys=True)


# --------------------------------------------------------------------------
# test/StaticTest.jl binary (unitless, G = 1)
# --------------------------------------------------------------------------
def binary_static():
    G, M, D, h, eta = 1.0, 1.0e10, 2.0, 1.0e-4, 0.025
    v = math.sqrt(G * M / D / 2.0)                     # binary_rot_vel
    acc = G * M / (D * D + h * h) / math.sqrt(D * D + h * h) * D   # binary_force
    pot = -1.0 * G * M * M / math.sqrt(D * D + h * h)  # binary_potential (0.5 sum pot_i)
    kin = M * v * v                                    # binary_kinetic
    return {
        "G": G, "mass": M, "D": D, "softening": h, "eta": eta,
        "pos": [[0.5 * D, 0.0, 0.0], [-0.5 * D, 0.0, 0.0]],
        "vel": [[0.0, v, 0.0], [0.0, -v, 0.0]],
        "acc_abs": acc, "potential": pot, "kinetic": kin, "energy": pot + kin,
        "momentum": [0.0, 0.0, 0.0], "angular_momentum": [0.0, 0.0, M * v * D],
        "dt_bound": math.sqrt(2.0 * eta * h / acc),
        "rtol": math.sqrt(2.0 ** -52),  # Julia isapprox default rtol = sqrt(eps(Float64))
    }


# --------------------------------------------------------------------------
# test/StaticTest.jl box
# --------------------------------------------------------------------------
def spline_force(dp, m, G, h):
    r2 = dp[0] * dp[0] + dp[1] * dp[1] + dp[2] * dp[2]
    r = math.sqrt(r2)
    if r >= h:
        fac = m / (r2 * r)
    else:
        u = r / h
        h3 = 1.0 / h ** 3
        if u < 0.5:
            fac = m * h3 * (10.666666666667 + u * u * (32.0 * u - 38.4))
        else:
            fac = m * h3 * (21.333333333333 - 48.0 * u + 38.4 * u * u - 10.666666666667 * u ** 3
                            - 0.066666666667 / u ** 3)
    return [d * fac * G for d in dp]


def spline_pot(dp, m, G, h):
    r = math.sqrt(dp[0] ** 2 + dp[1] ** 2 + dp[2] ** 2)
    if r == 0.0:
        return 0.0
    if r >= h:
        return -m / r * G
    u = r / h
    if u < 0.5:
        wp = -2.8 + u * u * (5.333333333333 + u * u * (6.4 * u - 9.6))
    else:
        wp = -3.2 + 0.066666666667 / u + u * u * (10.666666666667 + u * (-16.0 + u * (9.6 - 2.133333333333 * u)))
    return m / h * wp * G


def box_probe():
    c = 1.9
    pts = [
        [+0.1 + c, +0.1 + c, +0.1 + c], [-0.1 + c, +0.1 + c, +0.1 + c],
        [+0.1 + c, -0.1 + c, +0.1 + c], [+0.1 + c, +0.1 + c, -0.1 + c],
        [-0.1 + c, -0.1 + c, +0.1 + c], [-0.1 + c, +0.1 + c, -0.1 + c],
        [+0.1 + c, -0.1 + c, -0.1 + c], [-0.1 + c, -0.1 + c, -0.1 + c],
        [+1.0, +1.0, +1.0], [-1.0, -1.0, -1.0],
    ]
    G, m, h = 1.0, 1.0e9, 1.0e-4
    probe = [0.0, 0.0, 0.0]
    fs = [spline_force([p[k] - probe[k] for k in range(3)], m, G, h) for p in pts]
    acc = [math.fsum(f[k] for f in fs) for k in range(3)]
    pot = math.fsum(spline_pot([p[k] - probe[k] for k in range(3)], m, G, h) for p in pts)
    return {"G": G, "mass": m, "softening": h, "pos": pts, "probe": probe, "acc": acc,
            "pot": pot, "rtol": math.sqrt(2.0 ** -52)}


# --------------------------------------------------------------------------
# test/Local-Timestep.jl circular binary, constant-step leapfrog
# --------------------------------------------------------------------------
def circular_binary_const_leapfrog():
    G, M, D, h, eta = 1.0, 1.0, 2.0, 1.0e-4, 0.025
    N = 2900
    vel = math.sqrt(G * M / D / 2.0)

    def compute_acc(x):
        r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2]
        nrm = math.sqrt(r2)
        s = -G * M / (4 * r2)
        return [s * (xi / nrm) for xi in x]

    def compute_dt(a):
        return math.sqrt(2 * eta * h / math.sqrt(a[0] ** 2 + a[1] ** 2 + a[2] ** 2))

    x = [0.5 * D, 0.0, 0.0]
    v = [0.0, vel, 0.0]
    a = compute_acc(x)
    dt = compute_dt(a)
    t = 0.0
    v = [v[k] + 0.5 * a[k] * dt for k in range(3)]
    for _ in range(N - 1):
        x = [x[k] + v[k] * dt for k in range(3)]
        a = compute_acc(x)
        v = [v[k] + a[k] * dt for k in range(3)]
        t = t + dt
    v = [v[k] - 0.5 * a[k] * dt for k in range(3)]
    return {"G": G, "mass": M, "D": D, "softening": h, "eta": eta, "N": N, "dt": dt,
            "time_end": t, "pos0": [[0.5 * D, 0.0, 0.0], [-0.5 * D, 0.0, 0.0]],
            "vel0": [[0.0, vel, 0.0], [0.0, -vel, 0.0]], "x_end": x[0], "y_end": x[1],
            "rtol": math.sqrt(2.0 ** -52)}


# --------------------------------------------------------------------------
# Adaptive integer time line for a 2-body system (pure Python restatement)
# --------------------------------------------------------------------------
def circular_binary_adaptive():
    G, M, D, h, eta = 1.0, 1.0, 2.0, 1.0e-3, 0.025
    TB = 1 << 30
    T0, T1 = 0.0, 1.0
    TI = (T1 - T0) / TB
    vel = math.sqrt(G * M / D / 2.0)
    pos = [[0.5 * D, 0.0, 0.0], [-0.5 * D, 0.0, 0.0]]
    v = [[0.0, vel, 0.0], [0.0, -vel, 0.0]]
    # slightly eccentric so the two bins evolve
    v[0][1] *= 0.9
    v[1][1] *= 0.9
    pos0 = [p[:] for p in pos]
    vel0 = [q[:] for q in v]
    beg = [0, 0]
    end = [0, 0]
    acc = [[0.0] * 3, [0.0] * 3]
    t_int = 0

    def force_all(active):
        for i in range(2):
            if not active[i]:
                continue
            j = 1 - i
            # sum over both sources in order (self term contributes zero)
            terms = []
            for jj in range(2):
                dp = [pos[jj][k] - pos[i][k] for k in range(3)]
                terms.append(spline_force(dp, M, G, h) if jj != i else [0.0, 0.0, 0.0])
            acc[i] = [terms[0][k] + terms[1][k] for k in range(3)]
            _ = j

    def get_ts(a):
        ac = math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])
        dt = math.sqrt(2 * eta * h / ac)
        ti = dt / TI
        tm = TB
        while tm > ti:
            tm >>= 1
        return tm

    force_all([True, True])
    for i in range(2):
        end[i] = get_ts(acc[i])
    for i in range(2):
        d = float(end[i] - beg[i])
        v[i] = [v[i][k] + acc[i][k] * 1.0 * 0.5 * d * TI for k in range(3)]
    steps = 0
    while True:
        mn = min(TB, min(end))
        last = t_int
        t_int = mn
        dt = float(t_int - last) * TI
        for i in range(2):
            pos[i] = [pos[i][k] + v[i][k] * dt for k in range(3)]
        active = [end[i] == t_int for i in range(2)]
        force_all(active)
        for i in range(2):
            if not active[i]:
                continue
            ti_step = get_ts(acc[i])
            if t_int == TB:
                ti_step = 0
            if TB - t_int < ti_step:
                ti_step = TB - t_int
            tstart = float(beg[i] + end[i]) / 2
            tend = float(end[i]) + 0.5 * float(ti_step)
            dtk = (tend - tstart) * TI
            v[i] = [v[i][k] + acc[i][k] * dtk for k in range(3)]
            beg[i] = end[i]
            end[i] = beg[i] + ti_step
        steps += 1
        if T0 + t_int * TI >= T1:
            break
    for i in range(2):
        d = float(end[i] - beg[i])
        v[i] = [v[i][k] + acc[i][k] * -1.0 * 0.5 * d * TI for k in range(3)]
    return {"G": G, "mass": M, "softening": h, "eta": eta, "time_base": TB, "time_begin": T0,
            "time_end": T1, "pos0": pos0, "vel0": vel0, "steps": steps, "pos": pos, "vel": v,
            "ti_begstep": beg, "ti_endstep": end, "rtol": 1e-12}


if __name__ == "__main__":
    w("binary_static.json", binary_static())
    w("box_probe.json", box_probe())
    w("circular_binary_const_leapfrog.json", circular_binary_const_leapfrog())
    w("circular_binary_adaptive.json", circular_binary_adaptive())
    print("written to", HERE)
