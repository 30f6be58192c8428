"""bench.py's reference arm on the host (no GPU): the JSON line of the DSMC
workload, and the unavailable line for workloads the arm does not time."""
import io
import json
import sys
from contextlib import redirect_stdout


def run_main(argv):
    import bench
    old = sys.argv
    sys.argv = ["bench.py"] + argv
    buf = io.StringIO()
    try:
        with redirect_stdout(buf):
            bench.main()
    finally:
        sys.argv = old
    return [json.loads(line) for line in buf.getvalue().splitlines() if line.startswith("{")]


def test_reference_arm_box_is_unavailable():
    (line,) = run_main(["--impl", "reference", "--config", "box21"])
    assert line["impl"] == "reference" and "unavailable" in line


def test_reference_arm_dsmc():
    (line,) = run_main(["--impl", "reference", "--config", "dsmc41", "--steps", "1", "--warmup", "0"])
    assert line["impl"] == "reference"
    assert line["config"]["workload"] == "dsmc41" and line["config"]["particles"] == 6_400_000
    assert line["value"] > 0 and line["unit"] == "particle-calls/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
