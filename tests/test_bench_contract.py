"""The benchmark's reference arm runs on the CPU and prints the one-line JSON
contract (metric, value, unit, timing keys, the CPU baseline and e2e)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--level",
                        "3", "--steps", "1", "--warmup", "0", "--cpu-targets", "64"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["unit"] == "Ginteractions/s"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0
    # the reference arm runs the oracle on the oracle's own inputs: no library
    # of the product is loaded
    libs = d["libraries_loaded_from_repo"]
    assert libs and all("/oracle/build/" in p for p in libs), libs
    assert not any("lpm_gb300" in p for p in libs)


def test_bench_arguments_parse():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True,
                       text=True, timeout=120, cwd=ROOT)
    assert r.returncode == 0
    for flag in ("--config", "--ff-theta", "--ff-rho-min", "--swe-level", "--no-learned"):
        assert flag in r.stdout


def _bench_module():
    import importlib.util

    spec = importlib.util.spec_from_file_location("lpm_bench", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_far_field_settings_are_valid():
    """The level-8 leg's settings: the configuration's own (learned, theta
    0.5) first, every form known, every rho_min inside [0, theta] (the far
    field rejects a larger one, and the expansion-only rows use 0.25), and at
    least one setting of each form."""
    b = _bench_module()
    form, theta, rho = b.C5_SETTINGS[0]
    assert (form, theta) == ("learned", 0.5)
    for form, theta, rho in b.C5_SETTINGS:
        assert form in b.NET_MODE
        assert 0.0 < theta <= 1.0
        used = rho if rho else 0.25
        assert 0.0 <= used <= theta, (form, theta, rho)
        assert (rho is None) == (form == "expansion_only")
    assert {f for f, _, _ in b.C5_SETTINGS} == set(b.NET_MODE)
