"""bench.py's reference arm runs on the CPU (the oracle on host cores): its JSON
line carries the fields the driver reads (no GPU needed)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", "0",
         "--steps", "1", "--warmup", "0"],
        cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["higher_is_better"] is False
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_cpu_leg_sample_and_json():
    """The default arm's cpu_baseline leg: a stratified sample in the
    reference's task order whose estimate and JSON object are well formed,
    and a workload below the sample size timed in full."""
    sys.path.insert(0, ROOT)
    import bench
    from gauxc_gb300 import workloads as W
    sd = W.config(0)["systems"][0]
    mol, basis, mg, lb = W.build_system(sd, device=False)
    _, infos = bench.host_stats(lb)
    total = sum(i["npts"] * i["nbe"] ** 2 for i in infos)
    pick, share, stride = bench.cpu_sample(infos, total / 4)
    assert stride == 4 and len(set(pick)) == len(pick)
    keys = [infos[i]["npts"] * infos[i]["nbe"] for i in pick]
    assert keys == sorted(keys, reverse=True)
    assert 0.1 < share < 0.5
    assert bench.cpu_sample(infos, total / 4)[0] == pick
    for work, full in ((total / 4, False), (bench.CPU_SAMPLE_WORK, True)):
        leg = bench.cpu_leg(basis, lb, mol, sd["P"], sd["functional"], work, infos)
        assert (leg["share"] >= 1.0) == full
        assert leg["est"] >= leg["dt"] > 0 and leg["fixed"] >= 0
        d = bench.cpu_baseline_dict(leg, leg["est"], 1, bench.sample_note(leg, leg["dt"]),
                                    leg["share"] < 1.0)
        assert json.loads(json.dumps(d))["extrapolated"] is (not full)
