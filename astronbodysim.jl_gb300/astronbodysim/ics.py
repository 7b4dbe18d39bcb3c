"""Seeded initial conditions: Plummer and truncated Hernquist spheres.

Plummer: radii by the inverse mass profile r = a / sqrt(u^(-2/3) - 1), isotropic
directions, speeds by von Neumann rejection on q^2 (1 - q^2)^(7/2) times the
local escape speed (Aarseth, Henon & Wielen 1974).  Hernquist (1990): radii by
the inverse of M(r) = M r^2 / (r + a)^2 truncated at r_max, speeds by rejection
sampling of v^2 f(E) with the isotropic Eddington distribution function of the
untruncated model.  Both are moved to the centre-of-mass frame.  Equal masses
M/N.  The reference's own generator (AstroIC.PlummerStarCluster) is an external
package that is not available; these generators are the input spec and both
the GPU path and the oracle always consume the same arrays.
"""
import numpy as np


def _isotropic(rng, n):
    c = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(1.0 - c * c)
    return np.stack([s * np.cos(phi), s * np.sin(phi), c], axis=1)


def _to_com(pos, vel, mass):
    mt = mass.sum()
    pos = pos - (mass[:, None] * pos).sum(0) / mt
    vel = vel - (mass[:, None] * vel).sum(0) / mt
    return pos, vel


def plummer(n, seed=0, G=1.0, M=1.0, a=1.0, com=True):
    rng = np.random.default_rng(seed)
    u = rng.uniform(0.0, 1.0, n)
    u = np.where(u <= 0.0, np.finfo(float).tiny, u)
    r = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    pos = r[:, None] * _isotropic(rng, n)
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        x = rng.uniform(0.0, 1.0, todo.size)
        y = rng.uniform(0.0, 0.1, todo.size)
        ok = y < x * x * (1.0 - x * x) ** 3.5
        q[todo[ok]] = x[ok]
        todo = todo[~ok]
    vesc = np.sqrt(2.0 * G * M / a) * (1.0 + (r / a) ** 2) ** -0.25
    vel = (q * vesc)[:, None] * _isotropic(rng, n)
    mass = np.full(n, M / n)
    if com:
        pos, vel = _to_com(pos, vel, mass)
    return {"pos": pos, "vel": vel, "mass": mass}


def _hernquist_df(E, G, M, a):
    """Isotropic f(E) of the Hernquist model for bound E < 0."""
    vg = np.sqrt(G * M / a)
    q = np.sqrt(np.clip(-E * a / (G * M), 0.0, 1.0 - 1e-12))
    q2 = q * q
    num = 3.0 * np.arcsin(q) + q * np.sqrt(1.0 - q2) * (1.0 - 2.0 * q2) * (8.0 * q2 * q2 - 8.0 * q2 - 3.0)
    return M / (8.0 * np.sqrt(2.0) * np.pi ** 3 * a ** 3 * vg ** 3) * num / (1.0 - q2) ** 2.5


_ENV_CACHE = {}


def _hernquist_envelope_table(G, M, a):
    """max over v of v^2 f(Phi + v^2/2) tabulated against psi = -Phi a / (G M)
    in (0, 1); depends only on the model's units, so it is computed once."""
    key = (G, M, a)
    if key not in _ENV_CACHE:
        # dense towards psi -> 0 (outskirts) and psi -> 1 (centre, where f(E)
        # diverges); the table stops 1e-9 short of the singular point
        psi = np.unique(np.concatenate([np.geomspace(1e-7, 0.5, 500),
                                        1.0 - np.geomspace(1e-9, 0.5, 500)]))
        phi = -psi * G * M / a
        vesc = np.sqrt(-2.0 * phi)
        grid = np.linspace(0.0, 1.0, 2049)[1:-1]
        pmax = np.empty(psi.size)
        for k in range(0, psi.size, 100):
            v = vesc[k:k + 100, None] * grid[None, :]
            pmax[k:k + 100] = (v * v * _hernquist_df(phi[k:k + 100, None] + 0.5 * v * v, G, M, a)).max(1)
        _ENV_CACHE[key] = (psi, np.log(pmax))
    return _ENV_CACHE[key]


def hernquist(n, seed=0, G=1.0, M=1.0, a=1.0, rmax=100.0, com=True):
    rng = np.random.default_rng(seed)
    umax = (rmax / (rmax + a)) ** 2
    s = np.sqrt(rng.uniform(0.0, umax, n))
    r = a * s / (1.0 - s)
    pos = r[:, None] * _isotropic(rng, n)
    phi = -G * M / (r + a)
    vesc = np.sqrt(-2.0 * phi)
    # rejection envelope: tabulated maximum of p(v) = v^2 f(phi + v^2/2), with margin
    psi_t, logp_t = _hernquist_envelope_table(G, M, a)
    env = 1.3 * np.exp(np.interp(-phi * a / (G * M), psi_t, logp_t))
    speed = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        v = rng.uniform(0.0, 1.0, todo.size) * vesc[todo]
        y = rng.uniform(0.0, 1.0, todo.size) * env[todo]
        p = v * v * _hernquist_df(phi[todo] + 0.5 * v * v, G, M, a)
        ok = y < p
        speed[todo[ok]] = v[ok]
        todo = todo[~ok]
    vel = speed[:, None] * _isotropic(rng, n)
    mass = np.full(n, M / n)
    if com:
        pos, vel = _to_com(pos, vel, mass)
    return {"pos": pos, "vel": vel, "mass": mass}


def collision(n_each, seed=0, G=1.0, M=1.0, a=1.0, separation=20.0, rmax=100.0):
    """Two Hernquist spheres, centres `separation` apart on a parabolic approach
    (relative speed sqrt(2 G (2M) / separation)), in the centre-of-mass frame."""
    s1 = hernquist(n_each, seed=seed, G=G, M=M, a=a, rmax=rmax)
    s2 = hernquist(n_each, seed=seed + 1, G=G, M=M, a=a, rmax=rmax)
    vrel = np.sqrt(2.0 * G * (2.0 * M) / separation)
    off = np.array([0.5 * separation, 0.0, 0.0])
    dv = np.array([0.5 * vrel, 0.0, 0.0])
    pos = np.concatenate([s1["pos"] - off, s2["pos"] + off])
    vel = np.concatenate([s1["vel"] + dv, s2["vel"] - dv])
    mass = np.concatenate([s1["mass"], s2["mass"]])
    return {"pos": pos, "vel": vel, "mass": mass}
