"""The autotuner's host logic on CPU, with a fake engine and a fake timer:
refused configurations are skipped, the fastest one is installed last (after
the fastest one-lane configuration, which the library keeps for the
adjoint), the sample is restored before every launch and after tuning, and
the cache is written and then used without timing."""
import json

import pytest

torch = pytest.importorskip("torch")

from pfgpu import abi, autotune, generate  # noqa: E402
from pfgpu.network import default_options  # noqa: E402


class FakeEngine:
    def __init__(self, net):
        self.net = net
        self.installed = []
        self.current = None
        self.launches = 0
        self.dirty_at_launch = 0

    def set_launch_config(self, threads_per_block, blocks_per_sm, jac_in_shared, lanes_per_cell):
        # a library-like refusal: no shared Jacobian above 128 threads, no
        # groups of 8 lanes
        if (jac_in_shared and threads_per_block > 128) or lanes_per_cell == 8:
            return abi.PF_ERR_INVALID
        self.current = (threads_per_block, blocks_per_sm, jac_in_shared, lanes_per_cell)
        self.installed.append(self.current)
        return abi.PF_OK

    def rstep(self, state, dt, stats=False, order=None):
        self.launches += 1
        if float(state.a["pri_molal"][0, 0]) != self.reference:
            self.dirty_at_launch += 1
        state.a["pri_molal"].mul_(2.0)          # a step changes the state
        state.a["newton_its"].fill_(7)


def cost(cfg):
    tpb, bps, js, g = cfg
    # fastest overall: 4 lanes, 128 threads, 2 blocks/SM; fastest one-lane:
    # 96 threads, 3 blocks/SM, Jacobian in shared memory
    c = 10.0 + abs(tpb - 128) / 32.0 + abs(bps - 2) + (0.0 if g == 4 else 5.0)
    if g == 1:
        c = 12.0 + abs(tpb - 96) / 32.0 + abs(bps - 3) + (0.0 if js else 1.0)
    return c


def test_tune_picks_installs_restores_and_caches(tmp_path):
    net = generate.random_network(6, 18, 2, seed=5, options=default_options())
    st, _, _ = generate.random_cells(net, 300, seed=9)
    state = st.to("cpu")
    eng = FakeEngine(net)
    eng.reference = float(state.a["pri_molal"][0, 0])
    before = state.a["pri_molal"].clone()
    timed = []

    def timer(fn):
        fn()
        timed.append(eng.current)
        return cost(eng.current)

    cache = str(tmp_path / "cache.json")
    top, table = autotune.tune(eng, state, 3600.0, max_cells=128, reps=1, timer=timer,
                               device_name="fake GPU", cache_path=cache)
    assert top == dict(threads_per_block=128, blocks_per_sm=2, jac_in_shared=0, lanes_per_cell=4)
    assert eng.installed[-2:] == [(96, 3, 1, 1), (128, 2, 0, 4)]
    # every accepted candidate timed reps + 1 times, none refused one timed
    accepted = [c for c in autotune.candidates() if not ((c["jac_in_shared"] and c["threads_per_block"] > 128)
                                                          or c["lanes_per_cell"] == 8)]
    assert len(table) == len(accepted) and len(timed) == 2 * len(accepted)
    assert all(t[3] != 8 and not (t[2] and t[0] > 128) for t in timed)
    assert [r["ms"] for r in table] == sorted(r["ms"] for r in table)
    # the sample was pristine before every launch; the caller's state is untouched
    assert eng.dirty_at_launch == 0
    assert torch.equal(state.a["pri_molal"], before)
    saved = json.load(open(cache))
    key = autotune.network_key(eng, "fake GPU")
    assert saved[key]["best"] == top and saved[key]["cells"] == 128
    # a second call takes the cached configuration without timing anything
    n0 = eng.launches
    top2, _ = autotune.tune(eng, state, 3600.0, timer=timer, device_name="fake GPU", cache_path=cache)
    assert top2 == top and eng.launches == n0 and eng.installed[-1] == (128, 2, 0, 4)
    # another device name misses the cache
    assert autotune.network_key(eng, "other GPU") != key


def test_tune_refuses_when_nothing_is_accepted(tmp_path):
    net = generate.random_network(4, 12, 1, seed=3, options=default_options())
    st, _, _ = generate.random_cells(net, 50, seed=1)

    class NoneAccepted(FakeEngine):
        def set_launch_config(self, **kw):
            return abi.PF_ERR_INVALID

    eng = NoneAccepted(net)
    with pytest.raises(RuntimeError, match="no candidate"):
        autotune.tune(eng, st.to("cpu"), 3600.0, timer=lambda fn: 1.0, device_name="fake GPU",
                      cache_path=str(tmp_path / "c.json"))
