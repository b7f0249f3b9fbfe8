"""D3Q19 ensemble on the GPU.  FP64 instances must match the reference's
SerialSimulator (fixtures from tests/golden/gen_golden.py) within 1e-12 -
in fact bit for bit, the kernel uses the oracle's operation order without
fused multiply-adds; FP32 instances state their error against FP64."""
import hashlib
import os

import numpy as np
import pytest

import oracle
from libgeodecomp_gb300 import lgd, workloads

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name + ".npz"), allow_pickle=False)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_lbm_fp64_bit_exact_against_reference_L8():
    g = load("lbm_L8")
    with lgd.LbmEnsemble([int(g["L"])], [float(g["omega"])], lid=float(g["lid"]), precision=8) as e:
        e.step(int(g["steps"]))
        out = e.download(0)
    np.testing.assert_array_equal(out, g["out"])


def test_lbm_fp64_L24_golden():
    g = load("lbm_L24")
    with lgd.LbmEnsemble([int(g["L"])], [float(g["omega"])], lid=float(g["lid"]), precision=8) as e:
        e.step(int(g["steps"]))
        out = e.download(0)
    np.testing.assert_array_equal(out.reshape(-1)[g["sample_idx"]], g["sample"])
    assert sha(out) == str(g["sha256"])


@pytest.mark.parametrize("config", [(1, 128, 1), (3, 64, 2), (16, 128, 1), (4, 256, 8)])
def test_lbm_ensemble_uneven_sizes_match_oracle_any_launch_shape(config):
    edges = [5, 12, 2, 9, 17, 3]
    omegas = [1.0, 1.3, 1.9, 0.7, 1.55, 1.2]
    with lgd.LbmEnsemble(edges, omegas, lid=0.05, precision=8) as e:
        e.set_config(*config)
        e.step(11)
        for j, (L, om) in enumerate(zip(edges, omegas)):
            np.testing.assert_array_equal(e.download(j), oracle.lbm(L, 11, om, 0.05), err_msg=str(j))


def test_lbm_persistent_equals_looped_launches():
    edges, omegas = workloads.lbm_ensemble(12, seed=3, edge_min=4, edge_max=20)
    with lgd.LbmEnsemble(edges, omegas, precision=4) as a, lgd.LbmEnsemble(edges, omegas, precision=4) as b:
        a.step(7)
        b.step_looped(7)
        for j in range(len(edges)):
            np.testing.assert_array_equal(a.download(j), b.download(j))


@pytest.mark.parametrize("precision", [4, 8])
def test_lbm_memory_path_variants_identical(precision):
    edges, omegas = workloads.lbm_ensemble(10, seed=9, edge_min=3, edge_max=21)
    out = []
    for variant in (0, 1):
        with lgd.LbmEnsemble(edges, omegas, precision=precision) as e:
            e.set_variant(variant)
            e.step(9)
            out.append([e.download(j) for j in range(len(edges))])
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)
    if precision == 8:
        np.testing.assert_array_equal(out[0][4], oracle.lbm(int(edges[4]), 9, float(omegas[4]), 0.05))


def test_lbm_tuner_picks_a_valid_shape_and_reset_restores_rest_state():
    edges, omegas = workloads.lbm_ensemble(16, seed=4, edge_min=8, edge_max=24)
    with lgd.LbmEnsemble(edges, omegas, precision=4) as e:
        (ty, th, ct), ms = e.tune(trial_steps=2)
        assert ty >= 1 and th in (128, 256, 512) and ct >= 1 and ms > 0
        e.reset()
        e.step(5)
        got = e.download(3)
    ref = oracle.lbm(int(edges[3]), 5, float(omegas[3]), 0.05)
    assert np.max(np.abs(got - ref)) < 1e-6


def test_lbm_fp32_error_against_fp64():
    L, om = 32, 1.7
    with lgd.LbmEnsemble([L], [om], precision=4) as e:
        e.step(200)
        f32 = e.download(0)
    f64 = oracle.lbm(L, 200, om, 0.05)
    rel_l2 = np.linalg.norm(f32 - f64) / np.linalg.norm(f64)
    max_abs = np.max(np.abs(f32 - f64))
    # measured on GB300: rel-L2 2.4e-5, max-abs 8.5e-6 (L = 32, omega 1.7, 200 steps)
    assert rel_l2 < 1e-4 and max_abs < 1e-4, (rel_l2, max_abs)


def test_lbm_fp64_config_beyond_register_budget_is_rejected():
    with lgd.LbmEnsemble([6], [1.2], precision=8) as e:
        with pytest.raises(lgd.LGDError) as err:
            e.set_config(4, 1024, 1)
        assert err.value.code == lgd.ERR_INVALID


def test_lbm_upload_roundtrip_and_errors():
    with lgd.LbmEnsemble([6, 4], [1.2, 1.5], precision=8) as e:
        f = np.random.default_rng(0).random((19, 4, 4, 4))
        e.upload(1, f)
        np.testing.assert_array_equal(e.download(1), f)
        buf = np.zeros(19 * 64)
        with pytest.raises(lgd.LGDError) as err:
            lgd.check(lgd.lib().lgd_lbm_download(e._h, 2, lgd._ptr(buf), buf.nbytes))
        assert err.value.code == lgd.ERR_RANGE
    with pytest.raises(lgd.LGDError):
        lgd.LbmEnsemble([4], [2.5])


# ----------------------------------------------- two steps per launch
@pytest.mark.parametrize("shape,ctas", [(0, 1), (0, 2), (1, 1), (1, 3), (1, 4)])
@pytest.mark.parametrize("steps", [10, 11, 13])
def test_lbm_two_steps_per_launch_bit_identical_fp64(shape, ctas, steps):
    """Depth 2 (the first step's populations of a column and its rim in
    shared memory) equals single steps and the oracle bit for bit: uneven
    instances smaller and larger than a tile, edges that are not multiples
    of the tile, an odd step count ending with one single step."""
    edges = [5, 12, 2, 33, 17, 3, 40]
    omegas = [1.0, 1.3, 1.9, 0.7, 1.55, 1.2, 1.8]
    with lgd.LbmEnsemble(edges, omegas, lid=0.05, precision=8) as e:
        e.set_time_block(2, shape, ctas)
        before = e.launch_count()
        e.step(steps)
        assert e.launch_count() - before == steps // 2 + steps % 2
        assert e.time_block() == (2, shape, ctas)
        for j, (L, om) in enumerate(zip(edges, omegas)):
            np.testing.assert_array_equal(e.download(j), oracle.lbm(L, steps, om, 0.05), err_msg=str(j))


def test_lbm_two_steps_graph_replay_across_uneven_calls():
    """Calls of 3, 9, 6 and 4 steps: the four-step graph replays start from
    either buffer (an odd call leaves the ensemble on the other one), and a
    change of form or residency between calls rebuilds the graph."""
    edges = [9, 33, 4, 20]
    omegas = [1.1, 1.7, 0.9, 1.45]
    with lgd.LbmEnsemble(edges, omegas, lid=0.05, precision=8) as e:
        e.set_time_block(2, 1, 2)
        for n in (3, 9):
            e.step(n)
        e.set_time_block(2, 0, 1)
        for n in (6, 4):
            e.step(n)
        for j, (L, om) in enumerate(zip(edges, omegas)):
            np.testing.assert_array_equal(e.download(j), oracle.lbm(L, 22, om, 0.05), err_msg=str(j))


def test_lbm_two_steps_fp32_equal_single_steps_and_reference_L24():
    edges, omegas = workloads.lbm_ensemble(20, seed=5, edge_min=6, edge_max=70)
    with lgd.LbmEnsemble(edges, omegas, precision=4) as a, lgd.LbmEnsemble(edges, omegas, precision=4) as b:
        a.set_time_block(2, 1, 4)
        a.step(8)
        b.step(8)
        for j in range(len(edges)):
            np.testing.assert_array_equal(a.download(j), b.download(j))
    g = load("lbm_L24")
    with lgd.LbmEnsemble([int(g["L"])], [float(g["omega"])], lid=float(g["lid"]), precision=8) as e:
        e.set_time_block(2, 1, 1)
        e.step(int(g["steps"]))
        assert sha(e.download(0)) == str(g["sha256"])


def test_lbm_tuner_reports_depth_and_results_stay_exact():
    edges, omegas = workloads.lbm_ensemble(24, seed=6, edge_min=16, edge_max=48)
    with lgd.LbmEnsemble(edges, omegas, precision=8) as e:
        e.tune(trial_steps=2)
        depth, shape, ctas = e.time_block()
        assert depth in (1, 2) and shape in (0, 1) and ctas >= 1
        e.reset()
        e.step(7)
        np.testing.assert_array_equal(e.download(5), oracle.lbm(int(edges[5]), 7, float(omegas[5]), 0.05))
    with lgd.LbmEnsemble([6], [1.2], precision=8) as e:
        with pytest.raises(lgd.LGDError):
            e.set_time_block(3, 0, 1)
        with pytest.raises(lgd.LGDError):
            e.set_time_block(2, 2, 1)
