"""The benchmark's reference arm (`bench.py --impl reference`) on the host:
one JSON line with the contract's keys, the oracle port as its only
compute, no library of the GB300 package mapped, and ranks other than 0
exiting without work.  Runs without a GPU."""
from __future__ import annotations

import json
import os
import subprocess
import sys

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))

KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
        "impl", "cpu_baseline", "e2e"}


def _run(*extra, env=None):
    e = dict(os.environ)
    e.pop("RANK", None)
    e.pop("WORLD_SIZE", None)
    e.update(env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                           *extra], capture_output=True, text=True, timeout=300, env=e, cwd=ROOT)


def _lines(out):
    return [json.loads(ln) for ln in out.splitlines() if ln.startswith("{")]


def test_reference_arm_line():
    r = _run("--nx", "64", "--ny", "48", "--steps", "2", "--warmup", "1")
    assert r.returncode == 0, r.stderr
    lines = _lines(r.stdout)
    assert len(lines) == 1
    ln = lines[0]
    assert KEYS <= set(ln)
    assert ln["impl"] == "reference"
    assert ln["unit"] == "evals/s" and ln["higher_is_better"] is True
    assert ln["value"] > 0 and ln["steps"] == 2 and ln["warmup"] == 1
    assert abs(ln["ms_per_step"] - 1000.0 / ln["value"]) < 1e-6 * ln["ms_per_step"]
    assert ln["config"]["nx"] == 64 and ln["config"]["ny"] == 48 and ln["config"]["ndof"] == 12
    cb = ln["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == ln["value"]
    assert ln["e2e"] == {"value": ln["value"], "unit": "evals/s",
                         "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the oracle is mapped; the product library is not
    assert any("liboracle" in x for x in ln["libraries"])
    assert not any("gfmd_gb300" in os.path.basename(x) for x in ln["libraries"])


def test_reference_arm_unknown_kernel_is_unavailable():
    r = _run("--nx", "16", "--ny", "16", "--steps", "1", "--warmup", "0",
             "--kernel", "isotropic 1.0 0.3")
    assert r.returncode == 0, r.stderr
    (ln,) = _lines(r.stdout)
    assert ln["impl"] == "reference" and "unavailable" in ln


def test_reference_arm_ndof_override():
    r = _run("--nx", "32", "--ny", "32", "--steps", "1", "--warmup", "0",
             "--kernel", "isotropic 1.0 0.3", "--ndof", "3")
    assert r.returncode == 0, r.stderr
    (ln,) = _lines(r.stdout)
    assert ln["config"]["ndof"] == 3 and ln["value"] > 0


def test_reference_arm_other_ranks_exit_quietly():
    r = _run("--nx", "64", "--ny", "64", "--steps", "1", "--warmup", "0",
             env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr
    assert _lines(r.stdout) == []
