"""CPU check of bench.py's reference arm (--impl reference): it times the
oracle port of the reference's CPU direct sum on a bounded sample of the same
workload the native arm reports, and prints one JSON line of the contract."""
import json
import os
import subprocess
import sys

from conftest import REPO


def test_reference_arm_line_names_the_native_workload():
    n = 4096
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0", "--n", str(n), "--ref-targets", "256"],
                         capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["config"]["workload"] == "plummer_n%d_eps1e-3_spline_mixed_kdk_dt1e-4" % n
    assert line["higher_is_better"] is True and line["unit"] == "G interactions/s"
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
