"""bench.py's reference arm on the CPU: one bounded sample of the headline
workload through the CPU restatement, printed as the one JSON line the
benchmark contract asks for."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "dtype",
                "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["metric"] == "Gcell-updates/s" and d["unit"] == "Gcell-updates/s" and d["higher_is_better"]
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["nx"] == 4096 and d["config"]["ny"] == 2048


def test_reference_arm_parameters_equal_the_library_defaults():
    """bench.py builds the headline parameter block without the library (its
    reference arm runs no product code); it must be the library's own."""
    sys.path.insert(0, ROOT)
    import bench
    from fivonagi_gb300 import _abi

    got = bench.headline_params(exact=True).as_dict()
    want = _abi.default_params(_abi.FV_APP_FOCUSED_BEAM).as_dict()
    assert got == want
    assert bench.headline_params(exact=False).exact == 0


def test_reference_arm_loads_no_product_library():
    code = ("import sys, json; sys.argv=['bench.py', '--impl', 'reference', '--steps', '1']; "
            "import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print(json.dumps({'loaded': 'libfivonagi' in maps}))")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert json.loads(lines[-1]) == {"loaded": False}
    ref_line = json.loads(lines[0])
    sys.path.insert(0, ROOT)
    import bench
    assert ref_line["config"] == bench.headline_config(bench.headline_params())
