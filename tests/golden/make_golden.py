"""Generate the golden fixtures by running the reference vegasflow 1.4.0 itself.

Usage (development container only; the reference tree must be present):

    python tests/golden/make_golden.py REFERENCE_ROOT
    VEGASFLOW_REFERENCE=REFERENCE_ROOT python tests/golden/make_golden.py

(REFERENCE_ROOT is the reference project's top directory, the one holding
``src/vegasflow``.)

The reference's ``src/vegasflow`` modules are imported unmodified, with
``tfshim`` installed as ``tensorflow`` (TensorFlow is not available here), and
driven through their public API (``VegasFlow``, ``PlainFlow``, ``VegasFlowPlus``,
``run_integration``, ``refine_grid_per_dimension``, ``consume_array_into_indices``)
on uniforms injected from ``numpy.random.default_rng(11)``.  Every raw uniform
block the reference consumed is stored next to its outputs, so the tests replay
exactly the same inputs through the oracle and the GPU kernels.

Output: ``tests/golden/golden.npz`` (a few hundred KB), ``reference_grid.json``
(written by the reference's save_grid) and ``repo_grid.json`` (written by this
project's save_grid and read back by the reference's load_grid).  With
``--c2-precision`` it writes ``c2_precision.npz`` instead: the reference's
float64 and float32 (``VEGASFLOW_FLOAT=32``) runs of the 8-D Gaussian on the
same injected uniforms.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
_args = [a for a in sys.argv[1:] if not a.startswith("--")]
REF = _args[0] if _args else os.environ.get("VEGASFLOW_REFERENCE")
if not REF or not os.path.isdir(os.path.join(REF, "src", "vegasflow")):
    sys.exit("make_golden.py: give the reference project's root (holding src/vegasflow) as the "
             "argument or in VEGASFLOW_REFERENCE")

sys.path.insert(0, HERE)
import tfshim  # noqa: E402

sys.modules["tensorflow"] = tfshim
sys.path.insert(0, os.path.join(REF, "src"))

import vegasflow  # noqa: E402
from vegasflow import monte_carlo as mc  # noqa: E402
from vegasflow import vflow, vflowplus, plain, utils  # noqa: E402

tf = tfshim
OUT = {}
RAW = []      # raw uniform blocks consumed, in order
TAPS = []     # (x, w, ind[, segm]) returned by _generate_random_array
EVENTS = []   # per-chunk accumulables returned by _run_event


def _source(rng):
    def draw(shape):
        u = rng.random(shape)
        RAW.append(u.copy())
        return u
    return draw


_orig_gen = mc.MonteCarloFlow._generate_random_array


def _gen(self, n_events, *args):
    out = _orig_gen(self, n_events, *args)
    TAPS.append([np.array(o) for o in out])
    return out


mc.MonteCarloFlow._generate_random_array = _gen


def _wrap_run_event(cls):
    orig = cls._run_event

    def run(self, *a, **k):
        out = orig(self, *a, **k)
        EVENTS.append([np.array(o) for o in out])
        return out

    cls._run_event = run


for _cls in (vflow.VegasFlow, vflowplus.VegasFlowPlus, plain.PlainFlow):
    _wrap_run_event(_cls)


def symgauss(xarr, weight=None):
    """Normalised symmetric Gaussian, a = 0.1 (the configs' integrand)."""
    n_dim = xarr.shape[-1]
    a = tf.constant(0.1, dtype=tf.float64)
    pref = tf.pow(1.0 / a / np.sqrt(np.pi), n_dim)
    coef = tf.reduce_sum(tf.square((xarr - 1.0 / 2.0) / a), axis=1)
    return pref * tf.exp(-coef)


def quirky_gauss(xarr, weight=None):
    """The reference tests' integrand verbatim in behaviour (test_algs.py:27-36)."""
    n_dim = xarr.shape[-1]
    a = tf.constant(0.1, dtype=tf.float64)
    n100 = tf.cast(100 * n_dim, dtype=tf.float64)
    pref = tf.pow(1.0 / a / np.sqrt(np.pi), n_dim)
    coef = tf.reduce_sum(tf.range(n100 + 1))
    coef += tf.reduce_sum(tf.square((xarr - 1.0 / 2.0) / a), axis=1)
    coef -= (n100 + 1) * n100 / 2.0
    return pref * tf.exp(-coef)


def simple_prod(xarr):
    """test_misc.py:24-26."""
    return tf.reduce_prod(tf.transpose(xarr), axis=0)


def run_case(name, make, integrand, n_iter, seed=11, freeze_after=None, **compile_kw):
    RAW.clear()
    TAPS.clear()
    EVENTS.clear()
    tfshim.set_uniform_source(_source(np.random.default_rng(seed)))
    inst = make()
    inst.compile(integrand, **compile_kw)
    grids, hist = [], []
    n_ev_hist = []
    for it in range(n_iter):
        if freeze_after is not None and it == freeze_after:
            inst.freeze_grid()
        if hasattr(inst, "n_ev"):
            n_ev_hist.append(np.array(inst.n_ev).copy())
        res, sig = inst._run_iteration()
        hist.append((float(np.asarray(res)), float(np.asarray(sig))))
        if hasattr(inst, "divisions"):
            grids.append(np.array(inst.divisions).copy())
    final = vegasflow_final(hist)
    OUT[f"{name}/raw"] = np.concatenate([r.reshape(-1) for r in RAW])
    OUT[f"{name}/raw_shapes"] = np.array([r.shape for r in RAW], dtype=np.int64)
    OUT[f"{name}/history"] = np.array(hist)
    OUT[f"{name}/final"] = np.array(final)
    if grids:
        OUT[f"{name}/grids"] = np.stack(grids)
    if n_ev_hist:
        OUT[f"{name}/n_ev"] = np.stack(n_ev_hist)
    # taps of the first chunk of the first iteration
    OUT[f"{name}/x0"] = TAPS[0][0]
    OUT[f"{name}/w0"] = np.asarray(TAPS[0][1]).reshape(-1)
    if len(TAPS[0]) > 2:
        OUT[f"{name}/ind0"] = TAPS[0][2].astype(np.int32)
    # per-chunk accumulables of every chunk (first element res or ress)
    OUT[f"{name}/ev_res"] = np.array([np.sum(np.asarray(e[0])) for e in EVENTS])
    if len(EVENTS[0]) > 2 and np.asarray(EVENTS[0][2]).size:
        OUT[f"{name}/arr_res2_0"] = np.asarray(EVENTS[0][2])
    return inst


def vegasflow_final(hist):
    """Replays monte_carlo.py:712-732 on the recorded history."""
    aux_res = 0.0
    weight_sum = 0.0
    for res, sigma in hist:
        wgt = 1.0 / pow(sigma, 2)
        aux_res += res * wgt
        weight_sum += wgt
    return aux_res / weight_sum, np.sqrt(1.0 / weight_sum)


def grid_interchange(ref_inst):
    """Grid JSON files across the two implementations (vflow.py:271-347): the
    reference's save_grid writes ``reference_grid.json`` (its trained 4-D grid,
    which this project's load_grid must read back exactly); this project's
    save_grid writes ``repo_grid.json``, which the reference's load_grid reads --
    what it loaded is stored for the tests."""
    ref_inst.save_grid(os.path.join(HERE, "reference_grid.json"))
    sys.path.insert(0, REPO)
    from vegasflow_gb300 import VegasFlow as RepoVegas  # save/load run on the host device

    rng = np.random.default_rng(77)
    sub = np.linspace(0.0, 1.0, 51)
    warped = np.stack([np.array(vflow.refine_grid_per_dimension(tf._t(rng.random(50) ** 4), tf._t(sub)))
                       for _ in range(3)])
    mine = RepoVegas(3, 1000, verbose=False, device="cpu")
    mine.load_grid(numpy_grid=warped)
    repo_file = os.path.join(HERE, "repo_grid.json")
    mine.save_grid(repo_file)
    ref3 = vflow.VegasFlow(3, 1000, verbose=False)
    ref3.load_grid(file_name=repo_file)
    loaded = np.array(ref3.divisions)
    assert np.array_equal(loaded, warped)
    OUT["interchange/repo_grid"] = warped
    OUT["interchange/ref_loaded_repo_grid"] = loaded


# -- C2 precision comparator: the reference in float64 and in its float32 mode
C2P_N, C2P_ITERS, C2P_SEED = 10_000_000, 3, 11
# Raw uniforms are floored at C2P_FLOOR in every run of the comparator: in the
# reference's float32 mode a raw uniform below ~3e-8 gives u whose 1 - u rounds
# to 1, so xn = 50 and the gather of the bin's upper edge (vflow.py:67-71) reads
# index 51 of a 51-edge grid -- TensorFlow raises on the CPU.  At 1e7 x 8
# uniforms per iteration about two such draws occur per iteration.
C2P_FLOOR = 3e-8


def c2_raw_source(rng):
    return lambda shape: np.maximum(rng.random(shape), C2P_FLOOR)


def c2_precision_child(out_path):
    """One run of the reference (VEGASFLOW_FLOAT taken from the environment at
    import) on C2's injected uniforms: 8-D Gaussian a = 0.1, C2P_N events per
    iteration in the default 1e6-event chunks, C2P_ITERS trained iterations, the
    raw uniforms of every iteration drawn from default_rng(C2P_SEED) in order."""
    from vegasflow.configflow import DTYPE

    tfshim.set_uniform_source(c2_raw_source(np.random.default_rng(C2P_SEED)))

    def gauss(xarr, weight=None):
        a = tf.constant(0.1, dtype=DTYPE)
        pref = tf.cast(tf.pow(1.0 / 0.1 / np.sqrt(np.pi), 8), dtype=DTYPE)
        return pref * tf.exp(-tf.reduce_sum(tf.square((xarr - 0.5) / a), axis=1))

    inst = vflow.VegasFlow(8, C2P_N, verbose=False)
    inst.compile(gauss)
    hist, grids = [], []
    for _ in range(C2P_ITERS):
        res, sig = inst._run_iteration()
        hist.append((float(np.asarray(res)), float(np.asarray(sig))))
        grids.append(np.array(inst.divisions, dtype=np.float64))
    np.savez(out_path, history=np.array(hist), grids=np.stack(grids), dtype=str(np.dtype(DTYPE.as_numpy_dtype)))


def c2_precision():
    """Runs c2_precision_child in float64 and float32 processes and writes
    ``c2_precision.npz``: the reference's naive float32 form set beside its
    float64 result on the same raw uniforms."""
    import subprocess
    import tempfile

    out = {"n_events": np.int64(C2P_N), "iterations": np.int64(C2P_ITERS), "seed": np.int64(C2P_SEED),
           "raw_floor": np.float64(C2P_FLOOR)}
    with tempfile.TemporaryDirectory() as tmp:
        for bits in ("64", "32"):
            path = os.path.join(tmp, f"c2_{bits}.npz")
            env = dict(os.environ, VEGASFLOW_FLOAT=bits)
            subprocess.run([sys.executable, os.path.abspath(__file__), REF, f"--c2-child={path}"], env=env,
                           check=True)
            r = np.load(path)
            out[f"f{bits}/history"] = r["history"]
            out[f"f{bits}/grids"] = r["grids"]
            assert str(r["dtype"]) == ("float64" if bits == "64" else "float32"), r["dtype"]
    path = os.path.join(HERE, "c2_precision.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}")


def main():
    rng = np.random.default_rng(2024)

    # -- refine_grid_per_dimension (vflow.py:135-211) on assorted histograms
    cases = []
    sub = np.linspace(0.0, 1.0, 51)
    cases.append((rng.random(50), sub))
    cases.append((np.exp(-((np.arange(50) - 25.0) / 6.0) ** 2), sub))
    spiky = np.zeros(50)
    spiky[7] = 3.0
    spiky[8] = 1.0
    cases.append((spiky, sub))
    cases.append((np.ones(50), sub))
    sparse = rng.random(50) * (rng.random(50) < 0.3)
    warped = np.cumsum(rng.random(51))
    warped = (warped - warped[0]) / (warped[-1] - warped[0])
    cases.append((sparse, warped))
    cases.append((rng.random(50) ** 8 * 1e-12, warped))
    OUT["refine/in"] = np.stack([c[0] for c in cases])
    OUT["refine/sub"] = np.stack([c[1] for c in cases])
    OUT["refine/out"] = np.stack([np.array(vflow.refine_grid_per_dimension(tf._t(c[0]), tf._t(c[1])))
                                  for c in cases])

    # -- importance-sampling map on a trained-looking grid (vflow.py:93-126)
    n_dim = 4
    grid = np.stack([np.array(vflow.refine_grid_per_dimension(tf._t(rng.random(50) ** 3), tf._t(sub)))
                     for _ in range(n_dim)])
    rnds = tf._t(rng.random((3000, n_dim)) * (1 - 2e-8) + 1e-8)
    x, w, ind = vflow._generate_random_array(rnds, tf._t(grid))
    OUT["map/grid"] = grid
    OUT["map/rnds"] = np.asarray(rnds)
    OUT["map/x"] = np.asarray(x)
    OUT["map/w"] = np.asarray(w)
    OUT["map/ind"] = np.asarray(ind).astype(np.int32)

    # -- consume_array_into_indices (utils.py:17-44)
    vals = rng.random(997)
    idx = rng.integers(0, 50, size=997).astype(np.int32)
    OUT["consume/in"] = vals
    OUT["consume/idx"] = idx
    OUT["consume/out"] = np.asarray(utils.consume_array_into_indices(tf._t(vals), tf._t(idx.reshape(-1, 1)),
                                                                     tf._t(np.int32(50))))

    # -- full integrations through the public API
    inst4 = run_case("vegas4", lambda: vflow.VegasFlow(4, 2000, verbose=False), symgauss, 3)
    grid_interchange(inst4)
    run_case("vegas4_chunks", lambda: vflow.VegasFlow(4, 1500, events_limit=400, verbose=False),
             symgauss, 2)
    run_case("vegas2_quirky", lambda: vflow.VegasFlow(2, 1000, verbose=False), quirky_gauss, 3)
    xmin = np.array([-1.0, 0.25, 0.0])
    xmax = np.array([3.0, 3.5, 1.0])
    OUT["vegas_limits/xmin"] = xmin
    OUT["vegas_limits/xmax"] = xmax
    run_case("vegas_limits", lambda: vflow.VegasFlow(3, 1200, xmin=xmin, xmax=xmax, verbose=False),
             simple_prod, 2)
    run_case("vegas_freeze", lambda: vflow.VegasFlow(3, 1000, verbose=False), symgauss, 3,
             freeze_after=2)
    run_case("plain3", lambda: plain.PlainFlow(3, 1500, verbose=False), symgauss, 2)
    run_case("plus2", lambda: vflowplus.VegasFlowPlus(2, 2000, adaptive=False, verbose=False),
             symgauss, 2)
    run_case("plus3_adaptive", lambda: vflowplus.VegasFlowPlus(3, 4000, adaptive=True, verbose=False),
             symgauss, 3)

    # -- VEGAS+ stratification set-up (vflowplus.py:103-139) for assorted sizes
    strat = []
    for n_dim_, n_ev_, adapt in [(2, 10000, False), (2, 10000, True), (3, 4000, True), (4, 10000, False),
                                 (4, 20000, True), (6, 2000000, True), (6, 2000000, False),
                                 (5, 100000, True), (8, 1000000, False), (1, 5000, True),
                                 (14, 100000, True), (3, 100, False)]:
        inst = vflowplus.VegasFlowPlus(n_dim_, n_ev_, adaptive=adapt, verbose=False)
        strat.append([n_dim_, n_ev_, int(adapt), int(inst._adaptive), int(inst._n_strat),
                      int(inst._hypercubes.shape[0]), int(inst.min_neval_hcube), int(inst.n_events)])
    OUT["strat/table"] = np.array(strat, dtype=np.int64)

    path = os.path.join(HERE, "golden.npz")
    np.savez_compressed(path, **OUT)
    print(f"wrote {path}: {os.path.getsize(path) / 1024:.0f} KB, {len(OUT)} arrays, "
          f"vegasflow {vegasflow.__version__}")


if __name__ == "__main__":
    child = [a for a in sys.argv[1:] if a.startswith("--c2-child=")]
    if child:
        c2_precision_child(child[0].split("=", 1)[1])
    elif "--c2-precision" in sys.argv:
        c2_precision()
    else:
        main()
