"""Seeded worldline configurations and the workload definitions.

A worldline configuration here has the reference's array layouts
(Path::beads / nextLink / prevLink, include/path.h:164-165; Worm::beads,
include/worm.h:153): positions AoS [M][Ne][3], links [M][Ne][2] (-1 = none),
on flags [M][Ne], worm locators int32[8] (head, tail, special1, special2).

Initial configurations follow the workload description: uniform positions in
the periodic cube, every bead of a particle jittered by N(0, 2 lambda tau) per
coordinate around it, identity permutation, wrapped by the minimum-image rule
of Container::putInBC (include/container.h:50-54).  numpy's Philox generator
makes them reproducible from a seed on any host.
"""
import math

import numpy as np

HE4_MASS = 4.000264          # amu; lambda = 24.24 / m = 6.0596 K A^2 (constants.cpp:128)
LAMBDA_HE4 = 24.24 / HE4_MASS
DENSITY = 0.02186            # A^-3


def box_side(n, density=DENSITY):
    """Prism(density, N) side (src/container.cpp:84-90)."""
    return (1.0 * n / density) ** (1.0 / 3.0)


def put_in_bc(r, side):
    side = np.asarray(side, dtype=np.float64)
    return r - side * np.floor(r * (1.0 / side) + 0.5)


def even_slices(temperature, tau):
    """Setup::worldlines (src/setup.cpp:995-1003): M = int(1/(T tau) + EPS), made even."""
    m = int(1.0 / (temperature * tau) + 1.0e-7)
    if m % 2:
        m -= 1
    return m


def default_mbar(n, volume, lam, tau, m):
    """Update length Mbar (src/setup.cpp:1079-1104)."""
    ell = (1.0 * n / volume) ** (-1.0 / 3.0)
    mbar = int(ell * ell / (16 * lam * tau))
    if mbar < 2:
        mbar = 2
    elif mbar > m:
        mbar = m // 2
    if mbar % 2:
        mbar += 1
    return mbar


def seeded_worldlines(n, m, side, lam, tau, seed, extent=None):
    """Return dict(pos, next, prev, on, worm) for N closed worldlines."""
    ne = n if extent is None else extent
    rng = np.random.Generator(np.random.Philox(seed))
    side = np.broadcast_to(np.asarray(side, dtype=np.float64), (3,))
    centre = (rng.random((n, 3)) - 0.5) * side
    jit = rng.normal(0.0, math.sqrt(2.0 * lam * tau), size=(m, n, 3))
    pos = np.zeros((m, ne, 3))
    pos[:, :n, :] = put_in_bc(centre[None, :, :] + jit, side)
    nxt = np.full((m, ne, 2), -1, dtype=np.int32)
    prv = np.full((m, ne, 2), -1, dtype=np.int32)
    s = np.arange(m, dtype=np.int32)
    for p in range(n):
        nxt[:, p, 0] = (s + 1) % m
        nxt[:, p, 1] = p
        prv[:, p, 0] = (s - 1) % m
        prv[:, p, 1] = p
    on = np.zeros((m, ne), dtype=np.uint8)
    on[:, :n] = 1
    worm = np.full(8, -1, dtype=np.int32)
    return dict(pos=np.ascontiguousarray(pos), next=nxt, prev=prv, on=on, worm=worm)


def open_worm(cfg, head, tail):
    """Cut the link after `tail`'s predecessor chain: a simple open worldline
    with head=(s_h, p) and tail=(s_t, p) on one particle, used to exercise the
    worm factors (Worm::factor, src/worm.cpp:108-118).  Beads strictly between
    head and tail (going forward from head) are switched off."""
    c = {k: v.copy() for k, v in cfg.items()}
    (sh, ph), (st, pt) = head, tail
    m = c["pos"].shape[0]
    # switch off beads after head up to before tail
    s, p = int(c["next"][sh, ph, 0]), int(c["next"][sh, ph, 1])
    while not (s == st and p == pt):
        ns, np_ = int(c["next"][s, p, 0]), int(c["next"][s, p, 1])
        c["on"][s, p] = 0
        c["next"][s, p] = -1
        c["prev"][s, p] = -1
        s, p = ns, np_
    c["next"][sh, ph] = -1
    c["prev"][st, pt] = -1
    c["worm"] = np.array([sh, ph, st, pt, -1, -1, -1, -1], dtype=np.int32)
    return c


# ---------------------------------------------------------------------------
# Workloads (synthetic stand-ins with the reference benchmark's shapes)
# ---------------------------------------------------------------------------
TAU = 0.004


def workload_plain_small():
    """Plain worm PIMC, N=16, T=2 K (reference forces M even: M=124, tau=1/248)."""
    n, t = 16, 2.0
    m = even_slices(t, TAU)
    return dict(n=n, m=m, temperature=t, tau=1.0 / (m * t), side=box_side(n), lam=LAMBDA_HE4)


def workload_pair_action(rc_mode="box"):
    """Pair-action microbench: N=256, T=1 K, tau=0.004 -> M=250, GSF."""
    n, t = 256, 1.0
    m = even_slices(t, TAU)
    L = box_side(n)
    return dict(n=n, m=m, temperature=t, tau=1.0 / (m * t), side=L, lam=LAMBDA_HE4,
                rc=(L if rc_mode == "box" else 7.0))


def workload_isf():
    """F(q,tau): N=512, M=512, tau=0.004 (T = 1/(M tau))."""
    n, m = 512, 512
    return dict(n=n, m=m, temperature=1.0 / (m * TAU), tau=TAU, side=box_side(n), lam=LAMBDA_HE4)


def isf_qvectors(side, count=2048, qmax=4.0, seed=0):
    """Sample `count` integer lattice vectors n with |2 pi n / L| <= qmax
    uniformly (Philox seed), returned as (q [count,3], n [count,3])."""
    nmax = int(qmax * side / (2 * math.pi)) + 1
    g = np.arange(-nmax, nmax + 1)
    nx, ny, nz = np.meshgrid(g, g, g, indexing="ij")
    lat = np.stack([nx.ravel(), ny.ravel(), nz.ravel()], axis=1)
    qn = 2 * math.pi / side * lat
    keep = np.sqrt((qn ** 2).sum(1)) <= qmax
    lat = lat[keep]
    rng = np.random.Generator(np.random.Philox(seed))
    idx = rng.choice(len(lat), size=min(count, len(lat)), replace=False)
    sel = lat[np.sort(idx)]
    return (2 * math.pi / side) * sel.astype(np.float64), sel.astype(np.int32)


def workload_walkers(num=1024, seed=0, tau=TAU, nmin=8, nmax=128, tmin=1.0, tmax=4.0):
    """Batched walkers: N ~ U{nmin..nmax}, T ~ U[tmin,tmax], M even from T and tau
    (the reference forces M even), T reset to 1/(M tau), Mbar from setup.cpp."""
    rng = np.random.Generator(np.random.Philox(seed))
    n = rng.integers(nmin, nmax + 1, size=num).astype(np.int32)
    t = rng.uniform(tmin, tmax, size=num)
    m = np.array([2 * int(round(1.0 / (2.0 * ti * tau))) for ti in t], dtype=np.int32)
    t = 1.0 / (m * tau)
    side = np.array([box_side(int(k)) for k in n])
    mbar = np.array([default_mbar(int(k), s ** 3, LAMBDA_HE4, tau, int(mm))
                     for k, s, mm in zip(n, side, m)], dtype=np.int32)
    return dict(n=n, m=m, temperature=t, side=side, mbar=mbar, tau=tau, lam=LAMBDA_HE4)


def permute(cfg, cycles):
    """Close worldlines into exchange cycles: for each tuple (p0, p1, ...) of
    particles, the bead of p_k on the last slice links to the bead of
    p_{k+1} on slice 0 (cyclically), and the prev links follow."""
    c = {k: v.copy() for k, v in cfg.items()}
    m = c["pos"].shape[0]
    for cyc in cycles:
        for k, p in enumerate(cyc):
            q = cyc[(k + 1) % len(cyc)]
            c["next"][m - 1, p] = (0, q)
            c["prev"][0, q] = (m - 1, p)
    return c


def workload_gp(points=4096, num_ptcl=64, num_slices=64, seed=0, matern_nu=2.5):
    """A seeded synthetic Gaussian-process potential and bead positions.

    Training inputs uniform in the normalised cube [-1, 1]^3, coefficients
    (K^-1 Y) normal with a small scale, hyperparameters of the magnitudes a
    helium-surface fit has; positions uniform in a 14 A cell about the
    origin.  The workload of one external-potential call is the beads of a
    path, num_ptcl x num_slices points."""
    rng = np.random.Generator(np.random.Philox(seed))
    train = np.empty((points, 4))
    train[:, :3] = rng.uniform(-1.0, 1.0, size=(points, 3))
    train[:, 3] = rng.normal(0.0, 2.0e-3, size=points)
    params = dict(matern_nu=matern_nu, ell=[0.7, 1.9, 0.8], norm_offset=[0.0, 0.0, -0.1],
                  norm_scale=[7.0, 3.5, 7.0], standard_mean=9.0, standard_std=95.0, mean=21.0,
                  sigma2=750.0, side=[14.0, 14.0, 14.0], periodic=[1, 1, 1])
    pos = rng.uniform(-7.0, 7.0, size=(num_ptcl * num_slices, 3))
    return dict(training=train, params=params, pos=pos)
