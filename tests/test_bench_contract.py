"""The benchmark's output contract, checked without a GPU: the reference arm
prints one JSON line with the keys the contract asks for and the same
config block as the GPU arm; the roofline block follows its definition
(the algorithmic bytes of every update a launch performs over the launch's
time, per-pass bytes beside it); every workload has a config; the traffic
figures come from the committed ncu summaries."""
import json
import os
import subprocess
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_reference_arm_prints_the_contract_line():
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-3000:]
    line = json.loads(res.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"] == bench.workload_config("jacobi7_f64_512", types.SimpleNamespace(time_block=0), 1)
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


class FakeWorkload:
    units = 10 ** 8
    bytes_per_unit = 16

    def traffic_key(self):
        return "jacobi7_f64_512_tb2"


def test_roofline_counts_every_update_of_a_fused_launch():
    # 10 steps in 5 launches of 2 steps, 1 ms in all: 0.2 ms per launch
    r = bench.roofline_of(FakeWorkload(), 1.0, 10, 5, 6766.0, "measured")
    assert r["steps_per_launch"] == 2.0 and r["launch_ms"] == 0.2
    assert r["algorithmic_bytes_per_launch"] == 10 ** 8 * 16 * 2
    assert r["achieved"] == pytest.approx(10 ** 8 * 16 * 2 / 0.2e-3 / 1e9, rel=1e-3)
    assert r["frac"] == pytest.approx(r["achieved"] / 6766.0, rel=1e-3)
    assert r["per_pass_bytes"] == 10 ** 8 * 16 and r["frac_per_pass"] == pytest.approx(r["frac"] / 2, rel=1e-3)
    assert r["traffic"] == bench.profile_traffic("jacobi7_f64_512_tb2") > 0
    # one step per launch: no per-pass block
    r1 = bench.roofline_of(FakeWorkload(), 1.0, 5, 5, 6766.0, "measured")
    assert "per_pass_gbs" not in r1 and r1["steps_per_launch"] == 1.0


@pytest.mark.parametrize("name", bench.WORKLOAD_NAMES)
def test_every_workload_has_a_config_and_a_metric(name):
    args = types.SimpleNamespace(time_block=0, lbm_instances=512, lbm_edge_max=192, size=512)
    cfg = bench.workload_config(name, args, 1)
    assert cfg["workload"].split("_")[0] == name.split("_")[0] and cfg["parallelism"] == "single GPU"
    assert bench.workload_config(name, args, 4)["parallelism"].endswith("4 ranks")
    assert bench.METRICS.get(name, bench.JACOBI_METRIC)


def test_traffic_summaries_name_committed_profiles():
    with open(os.path.join(ROOT, "profiles", "ncu_traffic.txt")) as f:
        rows = [l.split() for l in f if l.strip() and not l.startswith("#")]
    assert rows
    for key, value, summary in rows:
        assert float(value) > 0
        assert os.path.exists(os.path.join(ROOT, "profiles", summary)), summary


def test_host_placement_without_a_gpu_node_binds_nothing():
    class NoDevice:
        class cuda:
            @staticmethod
            def current_device():
                raise RuntimeError("no GPU")

    bench._PLACEMENT = None
    try:
        pl = bench.host_placement(NoDevice)
        assert pl["gpu_node"] is None and pl["bound_to_gpu_node"] is False and pl["cpus"] is None
        assert pl["numa_nodes"] >= 0
    finally:
        bench._PLACEMENT = None


def test_host_placement_binds_to_the_gpu_node(tmp_path):
    """Two NUMA nodes that share this process's CPUs, the GPU's PCI
    function on the second: pinned buffers are allocated from that node's
    CPUs."""
    allowed = sorted(os.sched_getaffinity(0))
    if len(allowed) < 2:
        pytest.skip("needs two CPUs")
    half = len(allowed) // 2
    for i, cpus in enumerate((allowed[:half], allowed[half:])):
        d = tmp_path / "devices" / "system" / "node" / ("node%d" % i)
        d.mkdir(parents=True)
        (d / "cpulist").write_text(",".join(str(c) for c in cpus) + "\n")
    pci = tmp_path / "bus" / "pci" / "devices" / "0000:00:07.0"
    pci.mkdir(parents=True)
    (pci / "numa_node").write_text("1\n")

    class Props:
        pci_domain_id, pci_bus_id, pci_device_id = 0, 0, 7

    class FakeTorch:
        class cuda:
            @staticmethod
            def current_device():
                return 0

            @staticmethod
            def get_device_properties(dev):
                return Props()

    bench._PLACEMENT = None
    try:
        pl = bench.host_placement(FakeTorch, sysfs=str(tmp_path))
        assert pl["numa_nodes"] == 2 and pl["gpu_node"] == 1 and pl["bound_to_gpu_node"]
        assert pl["cpus"] == allowed[half:]
    finally:
        bench._PLACEMENT = None
