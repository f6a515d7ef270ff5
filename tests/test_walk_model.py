"""Float32 model of the projection kernel's walk (csrc/siddon_fast.cuh,
``trace_fast``): drift batches guarded by the batch bound and its margin,
resynchronisation, the exact closing step, exact short batches and single
steps.  Many rays at once in NumPy float32 (fma modelled through float64:
the product is exact there, the sum may round twice in rare cases, so this
is a model of the arithmetic, not a bit-exact copy).

What it checks, for every batch length the kernels are built with:
* no step reads outside the cube: when a step's voxel is read, every plane
  family has taken no more crossings than the last one inside the cube;
* the counts recovered after a drift batch equal the crossings taken;
* the segment lengths add up to the chord.
Ray sets: random directions, directions within 1e-7 .. 1e-3 rad of an axis or
a coordinate plane, rays parallel to a plane (a family never crossed), and
rays with two families crossing at exactly the same parameters (ties).  CPU
only."""
import numpy as np
import pytest

F = np.float32
EPS23 = F(1.1920929e-7)  # 2^-23


def fma(a, b, c):
    # 0 * inf (a family parallel to the planes) gives NaN here as on the GPU;
    # callers select those lanes away
    with np.errstate(invalid="ignore"):
        return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(F)


def make_rays(n_rays, seed, kind):
    """Per-ray walk frames: spacing pa, crossing d of count 0 (the one nearest
    the chord midpoint), counts m0 of the first crossing before it, exit
    crossing counts, entry parameter t0 and exit parameter texit, all as the
    kernel's set-up leaves them (float32, parameters from the midpoint)."""
    rng = np.random.default_rng(seed)
    n = rng.integers(8, 300, size=(n_rays, 3)).astype(np.float64)
    u = rng.normal(size=(n_rays, 3))
    rows = np.arange(n_rays)
    if kind == "near_axis":
        # one or two components 1e-7 .. 1e-3 of the others
        for _ in range(2):
            j = rng.integers(0, 3, n_rays)
            pick = rng.random(n_rays) < 0.7
            u[rows[pick], j[pick]] *= 10.0 ** rng.uniform(-7, -3, pick.sum())
    elif kind == "in_plane":
        u[rows, rng.integers(0, 3, n_rays)] = 0.0
    elif kind == "ties":
        u[:, 1] = u[:, 0]
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    P = rng.uniform(0.05, 0.95, size=(n_rays, 3)) * n
    if kind == "ties":
        # families 0 and 1 identical (direction component, start point, axis
        # length): they cross at exactly the same parameters
        n[:, 1] = n[:, 0]
        P[:, 1] = P[:, 0]
    with np.errstate(divide="ignore", invalid="ignore"):
        a0 = np.where(u != 0, (0.0 - P) / u, -np.inf)
        a1 = np.where(u != 0, (n - P) / u, np.inf)
    lo = np.minimum(a0, a1)
    hi = np.maximum(a0, a1)
    lo[u == 0] = -np.inf
    hi[u == 0] = np.inf
    a_in = lo.max(1)
    a_out = hi.min(1)
    a_mid = 0.5 * (a_in + a_out)
    x_in = P + a_in[:, None] * u
    iv = np.clip(np.floor(x_in), 0, n - 1)
    pos = u > 0
    q1 = np.where(pos, iv + 1, iv)                     # first plane crossed
    jexit = np.where(pos, n - q1, q1)                  # crossing that leaves the cube
    au = np.abs(u)
    with np.errstate(divide="ignore", invalid="ignore"):
        pa64 = np.where(u != 0, 1.0 / au, np.inf)
        # crossing j at plane q1 +- j: alpha_j = alpha_0 + j * pa
        alpha0 = np.where(u != 0, (q1 - P) / u, np.inf)
        m0 = np.clip(np.rint((a_mid[:, None] - alpha0) / pa64), 0, jexit)
    m0 = np.where(u != 0, m0, 0.0)
    with np.errstate(invalid="ignore"):
        d64 = np.where(u != 0, alpha0 + m0 * pa64 - a_mid[:, None], np.inf)
    pa = pa64.astype(F)
    d = d64.astype(F)
    mexit = (jexit - m0).astype(F)
    with np.errstate(invalid="ignore"):
        texit = np.where(u != 0, fma(mexit, pa, d), F(np.inf)).min(1).astype(F)
    t0 = (a_in - a_mid).astype(F)
    return dict(pa=pa, d=d, m0=m0.astype(F), jexit=jexit, texit=texit, t0=t0, inplane=(u == 0),
                chord=(texit.astype(np.float64) - t0.astype(np.float64)), n=n)


def walk(R, batch, short=4):
    """Run the kernel's control flow over all rays in lock step (rays that
    leave a phase wait for the others, like the lanes of a warp)."""
    pa, d = R["pa"], R["d"]
    nr = pa.shape[0]
    inf = F(np.inf)
    m = np.where(R["inplane"], F(0), -R["m0"]).astype(F)       # counts from the midpoint crossing
    with np.errstate(invalid="ignore"):
        t = np.where(R["inplane"], inf, fma(m, pa, d))
    taken = np.zeros((nr, 3))                                   # crossings taken since the entry
    cur = R["t0"].copy()
    tstop = R["texit"]
    guard = (R["n"].sum(1) + 2).astype(np.int64)
    margin = (F(batch + 3) * EPS23 * (-R["t0"])).astype(F)
    sumL = np.zeros(nr)
    bad = np.zeros(nr, bool)
    resync_bad = np.zeros(nr, bool)
    steps = np.zeros(nr, np.int64)

    def gather_check(act):
        # the voxel of this step: every family's index still inside the cube
        bad[act] |= np.any(taken[act] > R["jexit"][act], axis=1)

    def exact_step(act):
        tm = t[act].min(1)
        L = tm - cur[act]
        gather_check(act)
        sumL[act] += L
        steps[act] += 1
        adv = t[act] == tm[:, None]
        mm = m[act] + adv.astype(F)
        tt = np.where(adv, fma(mm, pa[act], d[act]), t[act])
        m[act] = mm
        t[act] = tt
        taken[act] += adv
        cur[act] = tm

    active = np.ones(nr, bool)
    while True:   # drift batches
        with np.errstate(invalid="ignore"):
            bnd = fma(m + F(batch - 2), pa, d).min(1)
        act = active & (guard >= batch) & (bnd + margin < tstop)
        if not act.any():
            break
        guard[act] -= batch
        org = cur[act]
        tl = (t[act] - org[:, None]).astype(F)
        cl = np.zeros(act.sum(), F)
        idx = np.nonzero(act)[0]
        for s in range(batch - 1):
            tm = tl.min(1)
            L = tm - cl
            gather_check(act)
            sumL[act] += L
            steps[act] += 1
            adv = tl == tm[:, None]
            tl = np.where(adv, tl + pa[act], tl).astype(F)
            taken[act] += adv
            cl = tm
        # resync: counts from the drifted crossings, exact crossings again
        with np.errstate(invalid="ignore", over="ignore"):
            mr = np.rint((((tl + org[:, None]).astype(F) - d[act]).astype(F) / pa[act]).astype(F)).astype(F)
        fin = ~R["inplane"][act]
        expect = (taken[act] - R["m0"][act]).astype(F)
        resync_bad[idx] |= np.any(fin & (mr != expect), axis=1)
        m[act] = np.where(fin, mr, m[act])
        t[act] = np.where(fin, fma(m[act], pa[act], d[act]), inf)
        # closing exact step, length from the local frame
        tm = t[act].min(1)
        L = (tm - org) - cl
        gather_check(act)
        sumL[act] += L
        steps[act] += 1
        adv = t[act] == tm[:, None]
        mm = m[act] + adv.astype(F)
        t[act] = np.where(adv, fma(mm, pa[act], d[act]), t[act])
        m[act] = mm
        taken[act] += adv
        cur[act] = tm
    if short > 1:
        while True:   # exact short batches under the same bound (no margin)
            with np.errstate(invalid="ignore"):
                bnd = fma(m + F(short - 2), pa, d).min(1)
            act = (guard >= short) & (bnd < tstop)
            if not act.any():
                break
            guard[act] -= short
            for _ in range(short):
                exact_step(act)
    while True:       # single steps while the walk is inside the cube
        act = (cur < tstop) & (guard > 0)
        if not act.any():
            break
        guard[act] -= 1
        exact_step(act)
    return dict(bad=bad, resync_bad=resync_bad, sumL=sumL, steps=steps, taken=taken)


@pytest.mark.parametrize("kind", ["random", "near_axis", "in_plane", "ties"])
@pytest.mark.parametrize("batch", [16, 24, 32, 48])
def test_drift_batches_stay_inside_the_cube(kind, batch):
    R = make_rays(3000, seed=batch * 7 + len(kind), kind=kind)
    ok = R["chord"] > 0
    for k in R:
        if isinstance(R[k], np.ndarray) and R[k].shape[:1] == ok.shape:
            R[k] = R[k][ok]
    out = walk(R, batch)
    assert not out["bad"].any(), "a step read outside the cube"
    assert not out["resync_bad"].any(), "resynchronised counts differ from the crossings taken"
    # the walk reaches the exit of every ray and its lengths add up to the chord
    rel = np.abs(out["sumL"] - R["chord"]) / np.maximum(R["chord"], 1e-30)
    assert rel.max() < 1e-5, rel.max()
    # no family goes past the crossing that leaves the cube
    assert np.all(out["taken"] <= R["jexit"] + 1)
    if kind == "ties":
        # the tied families cross together, one step for both crossings
        shared = np.minimum(out["taken"][:, 0], out["taken"][:, 1])
        assert np.all(out["taken"].sum(1) - out["steps"] >= shared - 1)
