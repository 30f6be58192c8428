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


def test_host_sphere_steps_measure_their_iterations():
    """The reference arm's whole host step (inject, threaded push + removal +
    deposit, serial Newton-PCG from the previous potential, computeEF) on a
    small sphere: it reports the iterations it ran, not an assumed count."""
    import bench
    cfg = dict(bench.CONFIGS["sphere64"])
    cfg.update(n=(17, 17, 33), np=20_000, mpw0=8000.0)
    P0 = bench.synthetic_state(cfg, cfg["np"], 1)
    r = bench.cpu_sphere_steps(cfg, P0, threads=2, steps=2, warmup=1)
    assert r["converged"] and r["newton"] >= 1 and r["pcg"] >= 1 and r["cold_pcg"] >= r["pcg"]
    assert r["seconds"] > 0 and 15_000 < r["n"] < 25_000


def test_host_sample_costs_are_positive():
    import bench
    cfg = dict(bench.CONFIGS["sphere64"])
    cfg.update(n=(17, 17, 33), np=20_000, mpw0=8000.0)
    c = bench.cpu_sample_costs(cfg, 20_000, threads=2)
    assert c["pd_per_particle"] > 0 and c["pcg_iter_s"] > 0 and 0.9 < c["survive"] <= 1.0
