"""GPU parity tests: libwoogpu.so against the CPU oracle on the same seeded inputs.

FP64 plain mode performs the reference's operations in the reference's order on both sides
(no contraction: --fmad=false on the GPU, -ffp-contract=off on the CPU) and sums contact
forces per particle in the order of the reference's deterministic pass
(ContactLoop.cpp:250-257). The tests therefore require BITWISE equality of positions,
velocities, forces, torques and of the contact set with its per-contact state, step after
step (particles with more than 64 contacts included: their slots are added one after the other
in slot order, component by component). Exception, with the tolerance written in the test:
  * node orientations (the quaternion update uses sin/cos, whose last bit may differ between
    the CUDA and the C library): |dq| <= 1e-14.
"""
import numpy as np
import pytest

from woodem_gb300 import scenes, _plan, _native

from helpers import brute_force_pairs, two_spheres

pytestmark = pytest.mark.gpu


def _oracle(A, threads=4):
    from oracle.oracle import Oracle
    return Oracle(A, threads=threads, deterministic=True)


def _gpu_nodes(S):
    S.sync()
    nd = S.dem._nodes.soa
    return {k: nd.col(k).copy() for k in ("pos", "ori", "vel", "angVel", "force", "torque")}


def _compare_nodes(g, o, shapes, nodes_of, heavy_ok=True):
    for k in ("pos", "vel", "angVel"):
        assert np.array_equal(g[k], o[k]), "%s differs (max abs %g)" % (k, np.max(np.abs(g[k] - o[k])))
    assert np.max(np.abs(g["ori"] - o["ori"])) <= 1e-14
    for k in ("force", "torque"):
        assert np.array_equal(g[k], o[k]), "%s differs (max abs %g)" % (k, np.max(np.abs(g[k] - o[k])))


def _compare_contacts(cg, co):
    assert np.array_equal(cg["id_lo"], co["id_lo"]) and np.array_equal(cg["id_hi"], co["id_hi"]), \
        "pair sets differ: %d gpu vs %d oracle" % (len(cg["id_lo"]), len(co["id_lo"]))
    assert np.array_equal(cg["real"], co["real"])
    assert np.array_equal(cg["id_a"], co["id_a"])
    for k in ("fglob", "local", "cpt"):
        assert np.array_equal(cg[k], co[k]), "contact %s differs (max abs %g)" % (k, np.max(np.abs(cg[k] - co[k])))
    r = cg["real"] != 0
    assert np.array_equal(cg["trsf"][r], co["trsf"][r])


def _run_pair(S, chunks, steps):
    A = _plan.compile_scene(S)
    O = _oracle(A)
    shapes = A.particles["shape"]
    nodes_of = A.particles["nodes"][:, 0]
    nfull = []
    for _ in range(chunks):
        S.run(steps)
        O.run(steps)
        g = _gpu_nodes(S)
        o = O.nodes()
        _compare_nodes(g, o, shapes, nodes_of)
        _compare_contacts(S._sim.contacts(), O.contacts())
        assert S._sim.stats().n_full_runs == O.stats().n_full_runs
        nfull.append(O.stats().n_full_runs)
    return nfull


def test_box_settle_bitwise(gpu_lib):
    """Box settle (walls, FrictPhys + IdealElPl, damping 0.2): 1500 spheres, 3000 steps."""
    S = scenes.box_settle_small(n=1500, seed=0)
    nfull = _run_pair(S, 10, 300)
    assert nfull[-1] > 20  # many collider full runs exercised


def test_box_settle_full_size_bitwise(gpu_lib):
    """The full 10 000-sphere box settle, 2000 steps, bitwise against the oracle."""
    S = scenes.box_settle(n=10000, seed=0)
    _run_pair(S, 4, 500)


def test_hertz_drum_bitwise(gpu_lib):
    """Rotating drum (facets with fakeVel, rotating wall caps, HertzPhys + Hertz DMT law)."""
    S = scenes.hertz_drum(n=4000, seed=1, diameter=0.3, length=0.12, div=41, axDiv=8, fill_fraction=0.3)
    nfull = _run_pair(S, 8, 250)
    assert nfull[-1] > 3


def test_pair_set_exact(gpu_lib):
    """Broad phase alone on the same positions: identical pair sets, equal to the brute-force
    closed-AABB overlap set filtered by the masks (InsertionSortCollider.cpp:52-58, Collision.cpp:19-41)."""
    S = scenes.hertz_drum(n=3000, seed=4, diameter=0.3, length=0.12, div=31, axDiv=6, fill_fraction=0.32)
    A = _plan.compile_scene(S)
    O = _oracle(A)
    O.collide_only()
    sim = _plan.Simulation(S)
    S._sim = sim
    L, h = sim.H.L, sim.H.h
    sim.H.check(L.wg_collide_only(h), "collide_only")
    cg = _plan.read_contacts(L, h, "wg")
    co = O.contacts()
    assert np.array_equal(cg["id_lo"], co["id_lo"]) and np.array_equal(cg["id_hi"], co["id_hi"])
    mn, mx = np.empty((A.n_particles, 3)), np.empty((A.n_particles, 3))
    L.wg_get_aabbs(h, _native.ptr(mn), _native.ptr(mx))
    mo, xo = O.aabbs(A.n_particles)
    assert np.array_equal(mn, mo) and np.array_equal(mx, xo)
    bf = brute_force_pairs(A, mn, mx)
    # facet-facet / wall-facet / wall-wall pairs are excluded by the boundary masks
    assert bf == set(zip(cg["id_lo"].tolist(), cg["id_hi"].tolist()))


@pytest.mark.parametrize("v0", [1, 1e-2, 1e-4])
def test_hertz_collision_time_gpu(v0, gpu_lib):
    """py/tests/hertz.py:29-46 on the GPU: collision time within 1% of 2.214 (rho/E*)^(2/5) d v0^(-1/5)."""
    r = 0.05
    tau = 2.214 * (1e3 / (1e8 / (2 * (1 - .2 ** 2)))) ** 0.4 * (2 * r / v0 ** 0.2)
    S = two_spheres(gap=1e-12, v0=v0, r=r, hertz=True, dt=tau / 1000.0)
    n_real, started = 0, False
    for _ in range(5000):
        S.run(1)
        real = S._sim.stats().n_real
        if real:
            started = True
            n_real += 1
        elif started:
            break
    sim = n_real * S.dt
    assert abs(sim - tau) <= 0.01 * sim


def test_errors_are_raised(gpu_lib):
    """Unsupported engine lists and NaN states raise instead of running."""
    from woodem_gb300 import utils
    S = scenes.box_settle_small(n=50, seed=0, precision="fp32")
    S.engines = utils.defaultEngines(damping=.2)
    S.engines[0].reset = False  # Leapfrog without the force reset is outside the GPU path
    with pytest.raises(NotImplementedError):
        S.run(1)
    S = scenes.box_settle_small(n=50, seed=0)
    S.dem.par[10].pos = (float("nan"), 0, 0)
    with pytest.raises(RuntimeError):
        S.run(2)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_call_granularity_is_invisible(prec):
    """The step loop queues steps in chunks and resumes after each collider run; running 400 steps
    in one call, in calls of 1 and 37 steps, or through wg_run_host (state copied out and back in
    every call, from pageable or page-locked arrays; with page-locked arrays the kinematic state
    is copied out while the last contact loop of the call runs), one step or five steps per call,
    gives bitwise the same state, and the arrays hold the state wg_get_nodes reads after the call."""
    out = []
    for mode in ("one", "steps", "host", "pinned", "pinned5"):
        S = scenes.box_settle_small(n=1200, seed=5, precision=prec)
        if mode == "one":
            S.run(400)
        elif mode == "steps":
            S.run(1)
            for _ in range(10):
                S.run(37)
            for _ in range(29):
                S.run(1)
        else:
            S.run(1)
            sim = S._sim
            L, h = sim.H.L, sim.H.h
            na = sim.A.n_nodes
            pinned = None
            if mode == "host":  # pageable arrays: staged copies
                parts = [np.zeros(w * na) for w in (3, 4, 3, 3, 3, 3)]
            else:  # page-locked arrays (wg_host_alloc)
                import ctypes
                pinned = L.wg_host_alloc(19 * 8 * na)
                assert pinned
                buf = np.ctypeslib.as_array((ctypes.c_double * (19 * na)).from_address(pinned))
                cuts = np.cumsum([0, 3, 4, 3, 3, 3, 3]) * na
                parts = [buf[cuts[q]:cuts[q + 1]] for q in range(6)]
            sim.H.check(L.wg_get_nodes(h, *[_native.ptr(x) for x in parts]), "get_nodes")
            calls = [1] * 399 if mode != "pinned5" else [5] * 79 + [1] * 4
            for c in calls:
                sim.H.check(L.wg_run_host(h, c, *[_native.ptr(x) for x in parts]), "run_host")
            held = [x.copy() for x in parts]
            if pinned:
                L.wg_host_free(pinned)
        g = _gpu_nodes(S)
        if mode in ("host", "pinned", "pinned5"):
            for x, k in zip(held, ("pos", "ori", "vel", "angVel", "force", "torque")):
                if k != "ori":
                    assert np.array_equal(x.reshape(g[k].shape), g[k]), "%s: the arrays after wg_run_host (%s)" % (k, mode)
        S.close()
        out.append(g)
    for k in ("pos", "vel", "angVel", "force", "torque"):
        assert np.array_equal(out[0][k], out[1][k]), "%s: one call vs many" % k
        assert np.array_equal(out[0][k], out[2][k]), "%s: one call vs host round trips" % k
        assert np.array_equal(out[0][k], out[3][k]), "%s: one call vs round trips through page-locked arrays" % k
        assert np.array_equal(out[0][k], out[4][k]), "%s: one call vs five-step calls through page-locked arrays" % k


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_launch_shape_is_invisible(prec, gpu_lib):
    """Threads per contact block, the resident-grid sphere-sphere kernel (FP32-force mode),
    steps per chunk and CUDA-graph replay change only the speed: a box settle (IdealElPl, walls)
    and a drum (Hertz, facets, rotating walls) end bitwise the same under every launch shape."""
    from woodem_gb300 import tune
    shapes = [(0, 32, False, False), (128, 8, False, True), (-256, 32, True, False), (-256, 5, False, True)]
    for build in (lambda: scenes.box_settle_small(n=1200, seed=5, precision=prec),
                  lambda: scenes.hertz_drum(n=2500, seed=2, diameter=0.3, length=0.12, div=31, axDiv=6, fill_fraction=0.3,
                                            precision=prec)):
        out = []
        for shape in shapes:
            S = build()
            S.run(1)
            tune.set_launch(S._sim, *shape)
            S.run(499)
            out.append(_gpu_nodes(S))
            S.close()
        for q in range(1, len(shapes)):
            for k in ("pos", "vel", "angVel", "force", "torque"):
                assert np.array_equal(out[0][k], out[q][k]), "%s differs under launch shape %s" % (k, shapes[q])
