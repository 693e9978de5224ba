"""bench.py's reference arm on the host alone: the oracle prepares its own
inputs (constraint equilibration, initial auxvars) and times its RStep, so
the arm needs no GPU and runs no library kernel."""
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("config", ["c1"])
def test_reference_arm_line(config):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference",
                          "--config", config, "--steps", "1", "--warmup", "3"],
                         capture_output=True, text=True, timeout=600, env=env, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 3
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["cells"] == 1000 and d["config"]["step"].startswith("the second operator-split step")


def test_host_inputs_step_cleanly():
    """The host-built reference-arm cells are the first successes of the
    seeded draw, with positive molalities, and every one of them steps."""
    import numpy as np
    sys.path.insert(0, REPO)
    import bench
    net, st, o = bench.build_state_host("c1", 1000, 200)
    assert st.ncells == 200
    assert np.all(st.a["pri_molal"] > 0) and np.all(np.isfinite(st.a["sec_act_coef"]))
    o.rstep(net, st, 3600.0)
    assert np.all(st.a["status"] == 0) and np.all(st.a["newton_its"] > 0)


def test_reference_arm_config_matches_ours():
    """Both arms describe the workload with the same function, so their
    config objects agree key for key on the same workload."""
    sys.path.insert(0, REPO)
    import bench
    cfg = bench.workload("c2")
    a = bench.c2_config(cfg, 1_000_000, 86400.0, 1.12e9)
    b = bench.c2_config(cfg, 1_000_000, 86400.0, 1.12e9)
    assert a == b and set(a) == {"workload", "cells", "dt_s", "step", "l2"}


def test_newton_count_histogram_bins():
    """The bench line's Newton-count histogram: cells per bin [2^k, 2^(k+1)),
    a bin below 1 and an open last bin, every cell counted once."""
    import torch
    sys.path.insert(0, REPO)
    import bench
    its = torch.tensor([0, 1, 1, 2, 3, 4, 7, 8, 15, 16, 300, 511, 512, 1000], dtype=torch.int32)
    h = bench.its_histogram(its)
    assert h["bins"] == ["<1", "1-1", "2-3", "4-7", "8-15", "16-31", "32-63", "64-127", "128-255", "256-511",
                         ">=512"]
    assert h["cells"] == [1, 2, 2, 2, 2, 1, 0, 0, 0, 2, 2]
    assert sum(h["cells"]) == its.numel()
