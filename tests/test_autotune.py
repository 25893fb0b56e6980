"""Launch configurations (fgb_step_desc.cfg) and the autotuner.

The knobs only change how work is split among blocks, so every configuration
must give bit-identical FP64 results; the autotuner must return a configuration
made of allowed values and leave the tracer fields as it found them.
"""
import numpy as np
import pytest

from fesom2_tracer_dwarf_gb300 import autotune


def test_candidates_cover_allowed_values():
    assert autotune.stage_candidates("hflux", 3) == [{0: 2}, {0: 4}, {0: 8}]
    lo = autotune.stage_candidates("lo", 4)
    assert len(lo) == 9 and {1: 4, 4: 4} in lo
    assert autotune.chunk_candidates(6) == [1, 2]
    assert autotune.chunk_candidates(5) == [1]
    up = autotune.stage_candidates("update", 2)
    assert all(set(c) == {3, 6} for c in up)
    r32 = autotune.stage_candidates("ratio", 4, "fp32")
    assert len(r32) == 12 and {2: 4, 5: 1} in r32 and {2: 2, 5: 3} in r32 and {2: 1, 5: 4} in r32
    assert {0: 2, 7: 1} in autotune.stage_candidates("hflux", 4, "fp32") and {9: 1} in autotune.stage_candidates(
        "hflux", 4, "fp32")
    lo32 = autotune.stage_candidates("lo", 4, "fp32")
    lo32s = autotune.stage_candidates("lo", 4, "fp32", wsplit=True)
    # the whole-column LO kernel is a candidate only without w_split
    assert {1: 4, 4: 3} in lo32 and all(c.get(4) != 3 for c in lo32s)
    assert len(lo32s) == 2 * (len(lo32) - 1) and {1: 2, 4: 1, 8: 1} in lo32s and {1: 2, 4: 1, 8: 0} in lo32s


def test_cache_file_round_trip(tmp_path):
    p = str(tmp_path / "sub" / "tune.json")
    autotune._save_file(p, {"k": {"cfg": [8, 4, 2, 1, 4, 2, 1, 0], "ms": {"lo": 1.0}}})
    assert autotune._load_file(p)["k"]["cfg"][1] == 4
    assert autotune._load_file(str(tmp_path / "missing.json")) == {}


torch = pytest.importorskip("torch")


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def _case(K, hor, ver, lim, precision="fp64"):
    from fesom2_tracer_dwarf_gb300 import engine, synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    m = Mesh(30, 26, 12, periodic=True, orient_left=True)
    rng = np.random.default_rng(12)
    vel, w = synthetic.streamfunction_flow(m, rng, 200.0, cfl=0.5)
    T = synthetic.random_field(m, rng, K)
    e = engine.TracerAdvection(m, K, precision, hor, ver, lim, copy_ab=True)
    e.set_tracers(T)
    e.set_velocity(vel, w)
    return e, T


CFGS = [
    [0] * 8,
    [2, 1, 1, 1, 1, 1, 1, 1],
    [4, 2, 4, 1, 2, 4, 1, 2],
    [8, 4, 2, 2, 4, 1, 2, 1],
    [2, 1, 2, 4, 4, 2, 4, 0],
    [4, 2, 2, 2, 1, 3, 3, 2],
    [2, 4, 1, 4, 2, 4, 2, 1],
]


@pytest.mark.gpu
@pytest.mark.parametrize("schemes", [("MUSCL", "QR4C", "FCT"), ("MFCT", "PPM", "FCT"), ("UPW1", "CDIFF", "NONE")])
def test_launch_configurations_give_identical_results(schemes):
    _gpu()
    K = 4
    out = []
    for cfg in CFGS:
        e, T = _case(K, *schemes)
        e.set_launch(cfg)
        e.step(200.0, 3)
        out.append(e.values())
    for cfg, v in zip(CFGS[1:], out[1:]):
        assert np.array_equal(v, out[0]), f"cfg {cfg} differs from the default by {np.abs(v - out[0]).max()}"


@pytest.mark.gpu
def test_autotune_returns_valid_config_and_restores_fields(tmp_path):
    _gpu()
    e, T = _case(4, "MUSCL", "PPM", "FCT", "fp32")
    before = e.values()
    res = autotune.tune(e, dt=200.0, reps=2, cache_path=str(tmp_path / "t.json"))
    assert not res["cached"]
    cfg = res["cfg"]
    tiled = cfg[9] == 1  # the tiled edge kernel has its own launch shape
    assert (cfg[0] == 0 and cfg[7] == 0) if tiled else (cfg[0] in autotune.EDGE_WARPS and cfg[7] in autotune.SLICES)
    assert all(c in autotune.NODE_WARPS for c in cfg[1:4])
    assert all(c in autotune.SLICES + (3, 4) for c in cfg[4:7])  # FP32: layers per lane per pass
    assert set(res["ms"]) == {"hflux", "lo", "ratio", "update"}
    assert np.array_equal(e.values(), before)
    again = autotune.tune(e, dt=200.0, cache_path=str(tmp_path / "t.json"))
    assert again["cached"] and again["cfg"] == cfg
    ref, _ = _case(4, "MUSCL", "PPM", "FCT", "fp32")
    e.step(200.0, 2)
    ref.step(200.0, 2)
    # FP32 kernels may contract multiply-adds differently per tracer-chunk
    # instantiation, so the tuned and default steps agree to FP32 rounding.
    a, b = e.values(), ref.values()
    assert np.abs(a - b).max() <= 1e-5 * max(1.0, np.abs(b).max())


@pytest.mark.gpu
@pytest.mark.parametrize("schemes", [("MUSCL", "PPM", "FCT"), ("UPW1", "QR4C", "NONE")])
def test_fp32_launch_configurations_agree(schemes):
    """FP32 form: block sizes and layers per lane change only the split of the
    work (and at most the compiler's contraction of a few multiply-adds)."""
    _gpu()
    out = []
    for cfg in CFGS:
        e, T = _case(4, *schemes, precision="fp32")
        e.set_launch(cfg)
        e.step(200.0, 3)
        out.append(e.values())
    scale = np.abs(out[0]).max()
    for cfg, v in zip(CFGS[1:], out[1:]):
        assert np.abs(v - out[0]).max() <= 1e-6 * scale, f"cfg {cfg}"
