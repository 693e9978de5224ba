"""Benchmark: operator-split cell chemistry solves per second on GB300.

Workload (default, --config c2): one synthetic network with 12 primary
species, 40 aqueous complexes and 6 kinetic minerals over 1,000,000 cells,
FP64, dt = 1 day, T ~ U[5, 60] C (non-isothermal logK), totals log10
U[-6, -2] with H+ by charge balance.  Inputs are generated and equilibrated on
the device (pf_equilibrate_constraint); the state (~1.1 GB) is far larger than
L2, and every step restarts from the same initial state (device-to-device
reset, inside the timed step).

One step = one pf_rstep over all cells (RStep for every cell: Newton, dt
cuts, kinetic-state update).  value = cells x steps / time.
  value        batched persistent kernel, inputs resident in HBM
  e2e          pf_rstep_host: host buffers, H2D + step + D2H inside the call
  plain_gpu    the plain one-thread-per-cell form on the same inputs
  cpu_baseline the CPU restatement of the reference (oracle) on the host cores
--impl reference times that CPU restatement alone, on inputs it prepares
itself on the host (the reference itself is Fortran on PETSc and cannot be
built here).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "pflotran-elm-interface_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "cell chemistry solves/s at 1e-10 rel. tol vs plain GPU; adjoint/forward time ratio"
UNIT = "cell-solves/s"
MUTABLE = ("total", "pri_molal", "pri_act_coef", "sec_act_coef", "sec_molal", "mnrl_volfrac",
           "mnrl_rate", "status", "newton_its", "num_substeps", "total_sorb", "ionx_ref_sorbed", "ln_act_h2o")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def workload(name):
    if name == "c5":
        return dict(workload="global-implicit assembly, 128x128x64 structured grid, 12 primaries / 40 complexes / "
                             "6 kinetic minerals, 7-point stencil, SeqBAIJ bs=12", cells=1_000_000, dt=86400.0)
    if name == "c1":
        return dict(workload="calcite 10x10x10 operator-split RStep (ncomp 3, 6 complexes, kinetic calcite)",
                    cells=1000, dt=3600.0)
    return dict(workload="synthetic network, 12 primaries / 40 complexes / 6 kinetic minerals, "
                         "operator-split RStep, non-isothermal", cells=1_000_000, dt=86400.0)


def build_state(cfg_name, ncells, device, seed=2026, keep_inputs=False):
    import torch

    from pfgpu import abi, generate
    from pfgpu.engine import ReactionEngine
    from pfgpu.network import CellState, default_options

    if cfg_name == "c1":
        net = generate.calcite_network()
        st, ct, cc = generate.calcite_cells(net, ncells + ncells // 20 + 64, seed=20261203)
    else:
        net = generate.random_network(12, 40, 6, seed=12, options=default_options(isothermal=0))
        st, ct, cc = generate.random_cells(net, ncells + ncells // 20 + 64, seed=seed)
    eng = ReactionEngine(net)
    dev = st.to(device)
    its = eng.equilibrate(dev, ct, torch.from_numpy(cc).to(device))
    good = torch.nonzero(its > 0).flatten()[:ncells]
    if good.numel() < ncells:
        raise RuntimeError("only %d of %d cells equilibrated" % (good.numel(), ncells))
    dev = dev.subset(good)
    # initial auxvars (condition_control.F90:1638-1649) then the step prelude
    # of pm_osrt.F90:115-153 (RTUpdateAuxVars, TIMESTEP activity update)
    dev.a["pri_act_coef"].fill_(1.0)
    dev.a["sec_act_coef"].fill_(1.0)
    dev.a["sec_molal"].zero_()
    eng.update_auxvars(dev, False)
    eng.update_auxvars(dev, True)
    eng.update_auxvars(dev, True)
    eng.update_auxvars(dev, False)
    eng.update_activity_coefs(dev)
    torch.cuda.synchronize()
    if keep_inputs:
        return net, eng, dev, (st, ct, cc)
    return net, eng, dev


def constraint_measure(net, eng, inputs, cpu=True, reps=3):
    """Constraint equilibration of the cells' initial conditions
    (pf_equilibrate_constraint: TOTAL for every component, charge balance on
    H+), timed on the device from the same host inputs, and the oracle's
    restatement on the host cores on a bounded sample."""
    import numpy as np
    import torch
    st, ct, cc = inputs
    cct = torch.from_numpy(cc).to("cuda")
    ms = []
    for k in range(reps + 1):
        dev = st.to("cuda")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        its = eng.equilibrate(dev, ct, cct)
        e1.record()
        torch.cuda.synchronize()
        if k:
            ms.append(e0.elapsed_time(e1))
    out = {"cells": st.ncells, "ms": float(np.min(ms)), "cells_per_s": st.ncells / (float(np.min(ms)) * 1e-3),
           "newton_its_mean": float(its.to(torch.float64).clamp(min=0).mean()),
           "failed": int((its <= 0).sum())}
    if cpu:
        from oracle.oracle import Oracle
        o = Oracle()
        cores = os.cpu_count() or 1
        n = min(st.ncells, 50_000)
        sub = st.subset(np.arange(n))
        t = time.perf_counter()
        o.equilibrate(net, sub, ct, cc[:, :n] if cc.ndim == 2 else cc, nthreads=cores)
        el = time.perf_counter() - t
        out["cpu_baseline"] = {"value": n / el, "unit": "cells/s", "cores": cores, "kind": "port",
                               "sample": "%d cells, %.2f s" % (n, el)}
    return out


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        import tempfile
        self.index = index
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="pfgpu_clocks_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(", ") for r in open(self.path).read().strip().splitlines()]
        except Exception:
            return None
        try:
            os.unlink(self.path)
        except OSError:
            pass
        rows = [r for r in rows if len(r) >= 8]
        if not rows:
            return None
        sm = sorted(float(r[0]) for r in rows)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[4:8]):
                if v.strip() == "Active":
                    reasons.add(nm)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": float(rows[0][1]), "reasons": sorted(reasons),
                "samples": len(rows)}


def fp64_peak(lib, device_sms, clocks=None):
    """Measured FP64 FMA throughput (TFLOP/s) with the library's probe.
    clocks: a dict that receives the SM clock nvidia-smi saw while the probe
    ran (a second of back-to-back launches), which the probe's fraction of
    the DFMA issue rate is read against."""
    import ctypes as C

    import torch
    blocks, threads, iters = device_sms * 8, 256, 5000
    out = torch.empty(blocks * threads, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()

    def launch(b=blocks, t=threads):
        lib.pf_bench_fp64_fma(C.c_void_p(out.data_ptr()), iters, b, t, C.c_void_p(s.cuda_stream))

    def rate(b, t):
        r = 0.0
        for _ in range(4):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            launch(b, t)
            e1.record()
            torch.cuda.synchronize()
            r = max(r, b * t * iters * 16.0 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
        return r
    best = rate(blocks, threads)
    if clocks is not None:
        # the same rate at a quarter and a sixteenth of the warps per SM: the
        # probe is not short of independent work
        clocks["shapes"] = {"64 warps/SM": best, "16 warps/SM": rate(device_sms * 2, threads),
                            "4 warps/SM": rate(device_sms, 128)}
        with Clocks(torch.cuda.current_device()) as clk:
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 1.2:
                for _ in range(8):
                    launch()
                torch.cuda.synchronize()
        clocks.update(clk.summary() or {})
    return best


STEP = ("the second operator-split step from the equilibrated state, its work queue in cell order (the first "
        "step, untimed, gives the state it starts from)")


def c2_config(cfg, ncells, dt, state_bytes):
    """The workload description both arms print (ours and --impl reference)."""
    if state_bytes > 129e6:
        l2 = "state %.2f GB > L2 (129 MB); state reset to the step's input before each timed step" % (state_bytes / 1e9)
    else:
        l2 = ("state %.1f MB fits in L2, not flushed: this small case is launch-bound; state reset before each "
              "timed step" % (state_bytes / 1e6))
    return {"workload": cfg["workload"], "cells": ncells, "dt_s": dt, "step": STEP, "l2": l2}


ITS_EDGES = (1, 2, 4, 8, 16, 32, 64, 128, 256, 512)


def its_histogram(its):
    """Cells per Newton-count bin [edge_k, edge_k+1) of a step's per-cell
    Newton iterations (a device int32 tensor); the last bin is open."""
    import torch
    edges = torch.tensor(ITS_EDGES, dtype=torch.int64, device=its.device)
    b = torch.bucketize(its.to(torch.int64), edges, right=True)
    counts = torch.bincount(b, minlength=len(ITS_EDGES) + 1).cpu().tolist()
    return {"bins": ["<1"] + ["%d-%d" % (lo, hi - 1) for lo, hi in zip(ITS_EDGES, ITS_EDGES[1:])] +
                    [">=%d" % ITS_EDGES[-1]],
            "cells": counts}


def time_steps(eng, dev, pristine, dt, kernel, steps, warmup, order=None):
    import torch
    from pfgpu import abi  # noqa: F401

    def reset():
        for k in MUTABLE:
            if k in dev.a:
                dev.a[k].copy_(pristine[k], non_blocking=True)

    for _ in range(warmup):
        reset()
        eng.rstep(dev, dt, kernel=kernel, stats=False, order=order)
    torch.cuda.synchronize()
    ks = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    for a, b in ks:
        reset()
        a.record()
        eng.rstep(dev, dt, kernel=kernel, stats=False, order=order)
        b.record()
    t1.record()
    torch.cuda.synchronize()
    total_ms = t0.elapsed_time(t1)
    kern_ms = [a.elapsed_time(b) for a, b in ks]
    return total_ms, kern_ms


def adjoint_measure(eng, dev, start, dt, order, reps, forward_ms):
    """pf_adjoint of one step from `start` (loss sum w*(T_final - target)^2,
    w ~ U[0,1], target = the forward output with 5 % lognormal noise): its
    time, which includes the recomputed forward solve, over forward_ms."""
    import numpy as np
    import torch
    for k in start:
        dev.a[k].copy_(start[k])
    eng.rstep(dev, dt, stats=False, order=order)
    gen = torch.Generator(device="cuda").manual_seed(4)
    w = torch.rand(dev.a["total"].shape, dtype=torch.float64, device="cuda", generator=gen)
    tgt = dev.a["total"] * torch.exp(0.05 * torch.randn(dev.a["total"].shape, dtype=torch.float64,
                                                         device="cuda", generator=gen))
    adj_ms = []
    for k_ in range(1 + reps):
        for k in start:
            dev.a[k].copy_(start[k])
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record()
        gout = eng.adjoint(dev, dt, weight=w, target=tgt, order=order)
        a1.record()
        torch.cuda.synchronize()
        if k_:
            adj_ms.append(a0.elapsed_time(a1))
    return {"ms": float(np.mean(adj_ms)), "forward_ms": forward_ms,
            "ratio_to_forward": float(np.mean(adj_ms)) / forward_ms,
            "cells_with_gradient": int((gout["adj_status"] == 0).sum()), "loss": float(gout["loss"][0])}


def cpu_baseline(net, host_state, dt, budget_s=15.0):
    """The oracle (C++ restatement of the reference, OpenMP over cells) on a
    bounded sample of the same cells, all host cores."""
    from oracle.oracle import Oracle
    o = Oracle()
    cores = os.cpu_count() or 1
    n = min(host_state.ncells, 2000)
    while True:
        sub = host_state.subset(range(n))
        t = time.perf_counter()
        o.rstep(net, sub, dt, nthreads=cores)
        el = time.perf_counter() - t
        if el > budget_s / 4 or n >= host_state.ncells:
            break
        n = min(host_state.ncells, int(n * min(8.0, max(2.0, (budget_s / 3) / max(el, 1e-3)))))
    return {"value": n / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d cells of the same workload, one RStep each, %.2f s" % (n, el)}


def girt_measure(net, eng, dev, steps, warmup, nx=128, ny=128, nz=64, seed=11, cpu=False):
    """Global-implicit residual + SeqBAIJ Jacobian assembly (pf_girt_assemble)
    on an nx*ny*nz structured grid with this network's cells (tiled over the
    grid), Darcy flux |q| ~ U[1e-7, 1e-5] m/s with random sign, D_m = 1e-9
    m^2/s, dt = 1 day.  The output (~nnzb*ncomp^2 doubles) is far larger than
    L2.  Two bounds: HBM (algorithmic bytes = each input read once + each
    output written once) and the FP64 pipe (flops of the assembly's
    arithmetic, flops.girt_per_cell)."""
    import numpy as np
    import torch

    from pfgpu.girt import GirtAssembler, StructuredGrid
    N = nx * ny * nz
    idx = torch.arange(N, device=dev.a["porosity"].device) % dev.ncells
    st = dev.subset(idx)
    rng = np.random.default_rng(seed)

    def q(shape):
        return rng.uniform(1e-7, 1e-5, shape) * rng.choice([-1.0, 1.0], shape)
    grid = StructuredGrid(nx, ny, nz, 1.0, 1.0, 1.0, q((nz, ny, nx - 1)), q((nz, ny - 1, nx)), q((nz - 1, ny, nx)),
                          diffusion=1e-9, tortuosity=1.0, dispersivity=0.0)
    asm = GirtAssembler(eng, grid)
    tk = (st.a["total"] * 1.01).contiguous()
    dt = 86400.0
    for _ in range(warmup):
        asm.assemble(st, tk, dt)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        a.record()
        asm.assemble(st, tk, dt)
        b.record()
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    # the later Newton iterations of a time step: each cell's K of every
    # reaction from the per-cell cache the step's first assembly filled
    asm.assemble(st, tk, dt, k_cache="fill")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        a.record()
        asm.assemble(st, tk, dt, k_cache="read")
        b.record()
    torch.cuda.synchronize()
    ms_read = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    n, ns, nm = net.ncomp, net.nsec, net.nmnrl
    nnzb = asm.nnzb
    # reads: pri_molal, pri/sec act coefs, volfrac, area, porosity, saturation,
    # volume, den, temperature, total_k, fluxes, pattern; writes: total,
    # sec_molal, mnrl_rate, residual, values
    rd = N * 8 * (n + n + ns + 2 * nm + 5 + n) + 8 * (grid.qx.size + grid.qy.size + grid.qz.size) + 4 * (N + 1 + nnzb)
    wr = N * 8 * (n + ns + nm + n) + nnzb * n * n * 8
    alg = rd + wr
    peak = None
    try:
        peak = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except Exception:
        pass
    gbs = alg / (ms * 1e-3) / 1e9
    from pfgpu import abi, flops
    fl, tr = flops.girt_per_cell(net, (nnzb - N) / N)
    tf = fl * N / (ms * 1e-3) / 1e12
    fp64 = fp64_peak(abi.load(), torch.cuda.get_device_properties(0).multi_processor_count)
    cpu_line = None
    if cpu:
        # the oracle's restatement of RTResidual/RTJacobian (one host core) on
        # a 32x32x16 block of the same cells
        from oracle.oracle import Oracle
        from pfgpu.girt import girt_pattern
        cx, cy, cz = 32, 32, 16
        Nc = cx * cy * cz
        host = st.subset(torch.arange(Nc, device=st.a["porosity"].device)).numpy()
        qh = {k: np.ascontiguousarray(v) for k, v in (("qx", q((cz, cy, cx - 1))), ("qy", q((cz, cy - 1, cx))),
                                                        ("qz", q((cz - 1, cy, cx))))}
        gd = dict(nx=cx, ny=cy, nz=cz, dx=1.0, dy=1.0, dz=1.0, diffusion=1e-9, tortuosity=1.0, dispersivity=0.0,
                  **qh)
        rp, ci = girt_pattern(cx, cy, cz)
        tkh = np.ascontiguousarray(host.a["total"] * 1.01)
        o = Oracle()
        t = time.perf_counter()
        o.girt_assemble(net, host, gd, tkh, dt, rp, ci)
        el = time.perf_counter() - t
        cpu_line = {"value": Nc / el, "unit": "cells/s", "cores": 1, "kind": "port",
                    "sample": "32x32x16 grid of the same cells, one assembly, %.3f s" % el}
    return {"grid": "%dx%dx%d" % (nx, ny, nz), "cells": N, "ncomp": n, "nnzb": nnzb, "ms": ms,
            "cpu_baseline": cpu_line,
            "cells_per_s": N / (ms * 1e-3), "algorithmic_bytes": alg, "achieved_gbs": gbs, "peak_gbs": peak,
            "hbm_frac": gbs / peak if peak else None, "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)",
            "flops_per_cell": fl, "transcendentals_per_cell": tr, "achieved_tflops": tf, "fp64_peak_tflops": fp64,
            "fp64_frac": tf / fp64 if fp64 else None, "kernels_per_assembly": 2,
            "k_cache_read": {"ms": ms_read, "cells_per_s": N / (ms_read * 1e-3),
                             "note": "later Newton iterations of a step: per-cell K (K/gamma of the complexes, "
                                     "K of the minerals) read from the cache the step's first assembly filled"}}


C3_NCOMP = (4, 6, 8, 10, 12, 16, 20, 24)


def build_c3(cells_per_network, device, seed=3000):
    """Eight networks generated like the 12/40/6 one with ncomp 4..24,
    3*ncomp complexes and ncomp/2 kinetic minerals; per-cell dt log-uniform
    in [1 h, 30 d]; cells equilibrated on the device."""
    import torch

    from pfgpu import generate
    from pfgpu.engine import ReactionEngine
    from pfgpu.network import default_options
    members = []
    for n in C3_NCOMP:
        net = generate.random_network(n, 3 * n, max(1, n // 2), seed=seed + n, options=default_options(isothermal=0))
        st, ct, cc = generate.random_cells(net, cells_per_network + cells_per_network // 10 + 64, seed=seed * 7 + n,
                                           dt_range=(3600.0, 30 * 86400.0))
        eng = ReactionEngine(net)
        dev = st.to(device)
        its = eng.equilibrate(dev, ct, torch.from_numpy(cc).to(device))
        good = torch.nonzero(its > 0).flatten()[:cells_per_network]
        if good.numel() < cells_per_network:
            raise RuntimeError("ncomp %d: only %d of %d cells equilibrated" % (n, good.numel(), cells_per_network))
        dev = dev.subset(good)
        dev.a["pri_act_coef"].fill_(1.0)
        dev.a["sec_act_coef"].fill_(1.0)
        dev.a["sec_molal"].zero_()
        eng.update_auxvars(dev, False)
        eng.update_auxvars(dev, True)
        eng.update_auxvars(dev, True)
        eng.update_auxvars(dev, False)
        eng.update_activity_coefs(dev)
        members.append((eng, dev))
    torch.cuda.synchronize()
    return members


def grid_dims(n):
    """(nx, ny, nz) with nx*ny*nz = n, as close to a cube as the divisors of n
    allow (nx >= ny >= nz)."""
    best = (n, 1, 1)
    z = 1
    while z * z * z <= n:
        if n % z == 0:
            m = n // z
            y = int(m ** 0.5)
            while y >= z and m % y:
                y -= 1
            if y >= z and max(m // y, y, z) < max(best):
                best = (m // y, y, z)
        z += 1
    return best


def transport_launches(stage):
    """Kernel launches of one fixed-schedule transport solve: coefficients,
    scaling, start copy, first residual; per cycle the inner start, five
    kernels per inner iteration, the FP64 update and residual; final copy."""
    return 4 + stage.refinements * (1 + 5 * stage.inner_iterations + 2) + 1


def c3_transport(members, seed=4000):
    """A structured grid per network (unit cells, Darcy flux U[1e-7, 1e-5]
    m/s with random sign, D_m = 1e-9 m^2/s), uniform dt = 1 day instead of
    the per-cell dt, and a fixed transport schedule from one adaptive step
    (taken on a copy of the totals)."""
    import numpy as np
    import torch

    from pfgpu.girt import StructuredGrid
    from pfgpu.network import CellState
    from pfgpu.timeloop import TransportStage
    from pfgpu.transport import OSTransport
    stages, info = [], []
    for i, (eng, dev) in enumerate(members):
        dev.a.pop("dt_cell", None)
        nx, ny, nz = grid_dims(dev.ncells)
        rng = np.random.default_rng(seed + i)

        def q(shape):
            return rng.uniform(1e-7, 1e-5, shape) * rng.choice([-1.0, 1.0], shape)
        grid = StructuredGrid(nx, ny, nz, 1.0, 1.0, 1.0, q((nz, ny, nx - 1)), q((nz, ny - 1, nx)),
                              q((nz - 1, ny, nx)), diffusion=1e-9, tortuosity=1.0, dispersivity=0.0)
        solver = OSTransport(grid, eng.net.ncomp)
        probe = CellState.__new__(CellState)
        probe.net, probe.ncells = dev.net, dev.ncells
        probe.a = {k: dev.a[k] for k in ("porosity", "saturation", "volume")}
        probe.a["total"] = dev.a["total"].clone()
        torch.cuda.synchronize()
        t = time.perf_counter()
        stats = solver.step(probe, 86400.0)
        torch.cuda.synchronize()
        inner, refs = OSTransport.schedule(stats)
        stages.append(TransportStage(solver, inner, refs))
        info.append(dict(ncomp=eng.net.ncomp, grid="%dx%dx%d" % (nx, ny, nz), adaptive_ms=1e3 * (time.perf_counter() - t),
                         adaptive_iterations=stats["iterations"], adaptive_refinements=stats["refinements"],
                         schedule=[inner, refs]))
    return stages, info


def c3_measure(args, per=500_000, nsteps=50, replays=1, plain=True, eager_steps=5):
    """Heterogeneous batching: 8 networks, per-cell dt, `nsteps` operator-split
    steps (RTUpdateAuxVars + TIMESTEP activities + RStep per network) in one
    CUDA graph; value = cells x steps / graph time.  The first step from the
    equilibrated state is also timed eagerly per network, batched against
    the plain one-thread-per-cell form."""
    import numpy as np
    import torch

    from pfgpu import abi, autotune
    from pfgpu.timeloop import OperatorSplitLoop
    t0 = time.perf_counter()
    members = build_c3(per, "cuda")
    log("c3 state built: %d x %d cells in %.1f s" % (len(members), per, time.perf_counter() - t0))
    stages = [None] * len(members)
    transport_info = None
    if getattr(args, "transport", False):
        stages, transport_info = c3_transport(members)
        log("c3 transport:", json.dumps(transport_info))
    tuned = {}
    for eng, dev in members:
        if args.no_tune:
            continue
        best, table = autotune.tune(eng, dev, 86400.0, max_cells=65536, reps=1, use_cache=False,
                                    quick=True, cost_order=True)
        tuned[eng.net.ncomp] = dict(best, ms_65k=table[0]["ms"])
    log("c3 autotune:", json.dumps(tuned))
    fields = [k for k in MUTABLE]
    start = [{k: dev.a[k].clone() for k in fields if k in dev.a} for _, dev in members]

    def reset(snap):
        for (_, dev), sn in zip(members, snap):
            for k, v in sn.items():
                dev.a[k].copy_(v)

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    # first step eagerly: per network, batched (natural order) vs plain
    per_net = []
    for i, (eng, dev) in enumerate(members):
        reset(start)
        b_ms = timed(lambda: eng.rstep(dev, 86400.0, stats=False))
        its = dev.a["newton_its"].to(torch.float64)
        p_ms = None
        if plain:
            reset(start)
            p_ms = timed(lambda: eng.rstep(dev, 86400.0, kernel=abi.PF_KERNEL_PLAIN, stats=False))
        per_net.append(dict(ncomp=eng.net.ncomp, nsec=eng.net.nsec, nmnrl=eng.net.nmnrl, cells=dev.ncells,
                            batched_ms=b_ms, plain_ms=p_ms, its_mean=float(its.mean()),
                            its_p50=float(its.median()), its_max=int(its.max()),
                            its_min=int(its.min())))
    batched_first = sum(r["batched_ms"] for r in per_net)
    plain_first = sum(r["plain_ms"] for r in per_net) if plain else None
    # the same first step as one persistent launch over every network's
    # cells (pf_rstep_multi), networks in descending ncomp
    from pfgpu.engine import rstep_multi
    by_cost = sorted(range(len(members)), key=lambda i: -members[i][0].net.ncomp)
    multi_ms = None
    if not getattr(args, "concurrent", False) and not getattr(args, "transport", False):
        reset(start)
        rstep_multi([members[i] for i in by_cost], 86400.0, stats=False)  # warm
        reset(start)
        multi_ms = timed(lambda: rstep_multi([members[i] for i in by_cost], 86400.0, stats=False))
    use_multi = multi_ms is not None and not getattr(args, "per_network", False)
    # one eager warm step of the loop (its Newton counts order the first graph step)
    reset(start)
    ordered = [members[i] for i in by_cost] if use_multi else members
    ordered_stages = [stages[i] for i in by_cost] if use_multi else stages
    loop = OperatorSplitLoop([(eng, dev, tr) for (eng, dev), tr in zip(ordered, ordered_stages)], dt=86400.0,
                             concurrent=getattr(args, "concurrent", False), multi=use_multi)
    loop.step()
    torch.cuda.synchronize()
    s0 = [{k: dev.a[k].clone() for k in fields if k in dev.a} for _, dev in members]
    loop.capture(nsteps)
    torch.cuda.synchronize()
    graph_ms = []
    with Clocks(0) as clk:
        for _ in range(max(1, replays)):
            reset(s0)
            graph_ms.append(timed(loop.replay))
    summary = loop.summary()
    eager_ms = None
    if eager_steps:
        k_e = min(nsteps, eager_steps)
        reset(s0)
        eager_ms = timed(lambda: [loop.step() for _ in range(k_e)]) / k_e
    total_cells = sum(dev.ncells for _, dev in members)
    g = float(np.min(graph_ms))
    value = total_cells * nsteps / (g * 1e-3)
    out = {"metric": "heterogeneous batched cell-solves/s, 8 networks, %d operator-split steps in one CUDA graph"
           % nsteps, "value": value, "unit": UNIT, "replays": len(graph_ms),
           "ms_per_step": g / nsteps,
           "config": {"workload": "8 synthetic networks ncomp %s, 3*ncomp complexes, ncomp/2 kinetic minerals, "
                                  "%d cells each, %s, T U[5,60] C" % (
                                      C3_NCOMP, per, "structured grid per network, transport solve + reaction "
                                      "each step, dt 1 d" if getattr(args, "transport", False)
                                      else "per-cell dt log-U[1 h, 30 d]"),
                      "graph_steps": nsteps, "concurrent_streams": bool(getattr(args, "concurrent", False)),
                      "l2": "state > L2; reset D2D before each replay, outside the timed region"},
           "graph_ms": g, "eager_ms_per_step": eager_ms,
           "first_step": {"batched_ms": batched_first, "plain_ms": plain_first,
                          "speedup_vs_plain_gpu": (plain_first / batched_first) if plain else None,
                          "one_launch_ms": multi_ms,
                          "one_launch_speedup_vs_plain_gpu": (plain_first / multi_ms) if (plain and multi_ms)
                          else None,
                          "per_network": per_net},
           "graph_reaction_step": "one persistent launch over all networks (pf_rstep_multi)" if use_multi
           else "one persistent launch per network",
           "last_step": summary, "autotune": tuned, "clocks": clk.summary(), "transport": transport_info,
           # per network per step: auxvars, activities, setup pre-pass, persistent kernel
           # (one persistent kernel for all with pf_rstep_multi; + the transport schedule's launches)
           "gpu_launches": len(graph_ms) * nsteps * ((3 * len(members) + 1) if use_multi else 4 * len(members)) +
           len(graph_ms) * nsteps * sum(transport_launches(tr) for tr in stages if tr is not None)}
    del members, loop, start, s0
    torch.cuda.empty_cache()
    return out


def run_c3(args):
    out = c3_measure(args, per=args.cells or 500_000, nsteps=args.graph_steps, replays=max(1, args.steps),
                     plain=True, eager_steps=5)
    line = {"metric": out.pop("metric"), "value": out.pop("value"), "unit": UNIT, "n_gpus": 1,
            "steps": out["replays"], "warmup": 1, "ms_per_step": out.pop("ms_per_step"), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": out.pop("config"), "gpu_launches": out.pop("gpu_launches")}
    line.update(out)
    print(json.dumps(line), flush=True)


def transport_measure(net, dev, steps, warmup, nx=128, ny=128, nz=64, seed=11, rtol=1e-10, cpu=False):
    """The transport half of the operator-split step (pf_transport_step) on
    the same grid as the global-implicit measurement: every component's
    totals transported over dt = 1 day to rtol by mixed-precision iterative
    refinement (FP32 Jacobi-BiCGStab corrections, FP64 residuals).
    Roofline: HBM; algorithmic bytes, per cell, with n components:
      inner FP32 iteration   76 n + 48  (the n-vectors read and written once
                             by the five kernels that use them: 19 floats;
                             the six scaled coefficients read by each of the
                             two stencil products)
      FP64 residual          24 n + 80  (x, T_k in, r out; 7 coefficients,
                             porosity, saturation, volume)
      refinement update      44 n + 8   (scaled start of the inner solve,
                             x += D^-1 y)
      set-up and copies      32 n + 200
    CPU baseline (cpu=True): the oracle's transport matrix (the restatement
    of RTCalculateTransportMatrix) and scipy's Jacobi-preconditioned BiCGStab
    per component to the same rtol, one host core, on a 32x32x16 grid of the
    same cells."""
    import numpy as np
    import torch

    from pfgpu.girt import StructuredGrid
    from pfgpu.network import CellState
    from pfgpu.transport import OSTransport
    N = nx * ny * nz
    idx = torch.arange(N, device=dev.a["porosity"].device) % dev.ncells
    src = dev.subset(idx)
    rng = np.random.default_rng(seed)

    def q(shape):
        return rng.uniform(1e-7, 1e-5, shape) * rng.choice([-1.0, 1.0], shape)
    grid = StructuredGrid(nx, ny, nz, 1.0, 1.0, 1.0, q((nz, ny, nx - 1)), q((nz, ny - 1, nx)), q((nz - 1, ny, nx)),
                          diffusion=1e-9, tortuosity=1.0, dispersivity=0.0)
    n = net.ncomp
    tr = OSTransport(grid, n)
    st = CellState.__new__(CellState)
    st.net, st.ncells = net, N
    st.a = {k: src.a[k] for k in ("porosity", "saturation", "volume")}
    t0 = src.a["total"].clone()
    st.a["total"] = t0.clone()
    dt = 86400.0
    for _ in range(warmup):
        st.a["total"].copy_(t0)
        stats = tr.step(st, dt, rtol=rtol)
    torch.cuda.synchronize()
    ms, its, refs = [], [], []
    for _ in range(steps):
        st.a["total"].copy_(t0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        stats = tr.step(st, dt, rtol=rtol)
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
        its.append(stats["iterations"])
        refs.append(stats["refinements"])
    t = float(np.mean(ms))
    it = float(np.mean(its))
    ref = float(np.mean(refs))
    alg = float(N) * ((76 * n + 48) * it + (24 * n + 80) * (ref + 1) + (44 * n + 8) * ref + 32 * n + 200)
    gbs = alg / (t * 1e-3) / 1e9
    peak = None
    try:
        peak = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except Exception:
        pass
    cpu_line = None
    if cpu:
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla

        from oracle.oracle import Oracle
        from pfgpu.girt import girt_pattern
        cx, cy, cz = 32, 32, 16
        Nc = cx * cy * cz
        crng = np.random.default_rng(seed + 1)

        def cq(shape):
            return crng.uniform(1e-7, 1e-5, shape) * crng.choice([-1.0, 1.0], shape)
        gd = dict(nx=cx, ny=cy, nz=cz, dx=1.0, dy=1.0, dz=1.0, diffusion=1e-9, tortuosity=1.0, dispersivity=0.0,
                  qx=cq((cz, cy, cx - 1)), qy=cq((cz, cy - 1, cx)), qz=cq((cz - 1, cy, cx)))
        por, sat, vol = (st.a[k][:Nc].cpu().numpy() for k in ("porosity", "saturation", "volume"))
        T = t0.reshape(n, -1)[:, :Nc].cpu().numpy()
        rp, ci = girt_pattern(cx, cy, cz)
        o = Oracle()
        tc = time.perf_counter()
        vals = o.transport_matrix(gd, por, sat, vol, dt, rp, ci)
        A = sp.csr_matrix((vals, ci, rp), shape=(Nc, Nc))
        psv = por * sat * 1000.0 * vol
        d = A.diagonal().copy()
        d[d == 0.0] = 1.0
        M = sp.diags(1.0 / d)
        for c in range(n):
            b = psv * T[c] / dt
            try:
                spla.bicgstab(A, b, x0=T[c].copy(), rtol=rtol, atol=0.0, M=M, maxiter=1000)
            except TypeError:
                spla.bicgstab(A, b, x0=T[c].copy(), tol=rtol, atol=0.0, M=M, maxiter=1000)
        el = time.perf_counter() - tc
        cpu_line = {"value": Nc / el, "unit": "cells/s", "cores": 1, "kind": "port",
                    "sample": "32x32x16 grid, %d components: oracle transport matrix + scipy Jacobi-BiCGStab to "
                              "rtol %g, %.3f s" % (n, rtol, el)}
    return {"grid": "%dx%dx%d" % (nx, ny, nz), "cells": N, "ncomp": n, "ms": t, "iterations": it, "refinements": ref,
            "cpu_baseline": cpu_line,
            "rel_residual": stats["max_rel_residual"], "rtol": rtol,
            "cells_per_s": N / (t * 1e-3), "algorithmic_bytes": alg, "achieved_gbs": gbs, "peak_gbs": peak,
            "hbm_frac": gbs / peak if peak else None, "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"}


def build_state_host(cfg_name, pool, nsample, seed=2026, nthreads=1):
    """The first nsample cells of build_state(cfg_name, pool, ...), prepared on
    the host by the oracle alone (constraint equilibration, initial auxvars,
    TIMESTEP activity update), so that no library kernel touches the
    reference arm's inputs and the arm runs without a GPU."""
    import numpy as np
    from pfgpu import generate
    from pfgpu.network import default_options
    from oracle.oracle import Oracle
    o = Oracle()
    if cfg_name == "c1":
        net = generate.calcite_network()
        st, ct, cc = generate.calcite_cells(net, pool + pool // 20 + 64, seed=20261203)
    else:
        net = generate.random_network(12, 40, 6, seed=12, options=default_options(isothermal=0))
        st, ct, cc = generate.random_cells(net, pool + pool // 20 + 64, seed=seed)
    # the same cells as the device build: equilibrate a prefix a little longer
    # than the sample and keep its first nsample successes, in order
    m = min(st.ncells, nsample + nsample // 10 + 64)
    st = st.subset(np.arange(m))
    _, its = o.equilibrate(net, st, ct, np.ascontiguousarray(cc[:, :m]), nthreads=nthreads)
    good = np.nonzero(its > 0)[0][:nsample]
    if good.size < nsample:
        raise RuntimeError("only %d of %d cells equilibrated" % (good.size, nsample))
    st = st.subset(good)
    st.a["pri_act_coef"][:] = 1.0
    st.a["sec_act_coef"][:] = 1.0
    st.a["sec_molal"][:] = 0.0
    for act in (False, True, True, False):
        o.update_auxvars(net, st, act, nthreads=nthreads)
    o.update_activity_coefs(net, st, nthreads=nthreads)
    return net, st, o


def run_reference(args):
    """The reference arm: the oracle (the C++ restatement of the reference's
    RStep; the Fortran reference needs PETSc and a Fortran compiler, neither
    present) on the host cores, on the same workload as our arm: the same
    generator and cells, prepared by the oracle itself, the first step
    untimed, then the second step timed over every cell."""
    import numpy as np  # noqa: F401
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg = workload(args.config)
    cores = os.cpu_count() or 1
    n = args.cells or cfg["cells"]
    name = "c2" if args.config == "c5" else args.config
    t0 = time.perf_counter()
    net, host, o = build_state_host(name, n, n, nthreads=cores)
    s1 = host.copy()
    o.rstep(net, s1, cfg["dt"], nthreads=cores)  # the first (untimed) step
    log("reference arm: %d cells prepared in %.1f s" % (n, time.perf_counter() - t0))
    state_bytes = sum(v.nbytes for v in s1.a.values())
    vals = []
    for k in range(args.warmup + args.steps):
        sub = s1.copy()
        t = time.perf_counter()
        o.rstep(net, sub, cfg["dt"], nthreads=cores)
        el = time.perf_counter() - t
        if k >= args.warmup:
            vals.append(n / el)
    v = float(np.median(vals)) if vals else 0.0
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n / v if v else None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": c2_config(cfg, n, cfg["dt"], state_bytes),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "every cell of the %d-cell workload, each step (median of %d steps)" % (
                                 n, len(vals))},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference is Fortran on PETSc (no Fortran compiler here); its C++ restatement timed"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c5"],
                    help="c3: 8 heterogeneous networks, time loop in one CUDA graph; "
                         "c5: only the global-implicit assembly on 128x128x64 cells")
    ap.add_argument("--graph-steps", type=int, default=50, help="c3: operator-split steps in the graph")
    ap.add_argument("--concurrent", action="store_true", help="c3: one stream per network inside the graph")
    ap.add_argument("--per-network", action="store_true",
                    help="c3: one persistent launch per network in the graph (default: one launch for all)")
    ap.add_argument("--transport", action="store_true",
                    help="c3: each network on a structured grid, transport solve before every reaction step "
                         "(uniform dt = 1 day)")
    ap.add_argument("--cells", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--no-girt", action="store_true")
    ap.add_argument("--no-c3", action="store_true", help="c2: leave out the heterogeneous-mix measurement")
    ap.add_argument("--c3-cells", type=int, default=0, help="c2: cells per network of the heterogeneous mix")
    ap.add_argument("--grid", default="128x128x64", help="global-implicit grid NXxNYxNZ")
    ap.add_argument("--launch", default="",
                    help="threads_per_block,blocks_per_sm,jac_in_shared[,lanes_per_cell] (skips tuning)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    import numpy as np
    import torch

    if args.impl == "reference":
        return run_reference(args)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from pfgpu import abi, flops
    if args.config == "c3":
        run_c3(args)
        return
    cfg = workload(args.config)
    ncells = args.cells or cfg["cells"]
    t_build = time.perf_counter()
    net, eng, dev, inputs = build_state("c2" if args.config == "c5" else args.config, ncells, "cuda",
                                        seed=2026 + rank, keep_inputs=True)
    log("state built: %d cells in %.1f s" % (ncells, time.perf_counter() - t_build))
    if args.config == "c5":
        nx, ny, nz = (int(v) for v in args.grid.split("x"))
        gm = None if args.no_girt else girt_measure(net, eng, dev, args.steps, args.warmup, nx, ny, nz,
                                                    cpu=not args.no_cpu)
        tm = transport_measure(net, dev, args.steps, max(2, min(args.warmup, 3)), nx, ny, nz,
                               cpu=rank == 0 and not args.no_cpu)
        if gm is None:
            gm = {"cells_per_s": float("nan"), "ms": float("nan")}
        if rank == 0:
            print(json.dumps({"metric": "global-implicit residual + SeqBAIJ Jacobian assemblies (cells/s)",
                              "value": gm["cells_per_s"] * world, "unit": "cells/s", "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": gm["ms"],
                              "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                              "data": "synthetic", "config": {"workload": cfg["workload"]}, "girt_assembly": gm,
                              "osrt_transport": tm,
                              "gpu_launches": 2 * args.steps}), flush=True)
        return
    s0 = {k: dev.a[k].clone() for k in MUTABLE if k in dev.a}
    dt = cfg["dt"]
    tuned = None
    if args.launch:
        vals = [int(x) for x in args.launch.split(",")]
        if eng.set_launch_config(*vals) != abi.PF_OK:
            raise SystemExit("launch config %s rejected" % args.launch)
    elif not args.no_tune:
        from pfgpu import autotune
        # the timed steps run with the queue in cell order: tune that way, on
        # a quarter of the cells
        best, table = autotune.tune(eng, dev, dt, use_cache=False, cost_order=False,
                                    max_cells=max(65536, ncells // 4), reps=1)
        tuned = {"best": best, "top": table[:6]}
        log("autotune:", json.dumps(tuned))

    # The timed step is the second operator-split step of a time loop: the
    # first step (untimed) takes the equilibrated state S0 to S1.  Its work
    # queue is in cell order: ordered by the first step's Newton counts
    # (descending, the only cost information a time loop has) it measured 2 %
    # slower -- the first step's stiff cells are not the second step's, and a
    # block's cells then come from all over the state, one 32-byte sector per
    # cell -- so that order is measured beside it (cost_order).
    # the first step itself, from the equilibrated state, in natural order (no
    # cost information exists yet), batched and plain
    nrep = max(1, min(args.steps, 3))
    f1_total, f1_kern = time_steps(eng, dev, s0, dt, abi.PF_KERNEL_BATCHED, nrep, 1)
    p1_total, p1_kern = time_steps(eng, dev, s0, dt, abi.PF_KERNEL_PLAIN, 1, 1)
    adjoint1 = adjoint_measure(eng, dev, s0, dt, None, nrep, float(np.mean(f1_kern)))
    for k in s0:
        dev.a[k].copy_(s0[k])
    stats1 = eng.rstep(dev, dt, kernel=abi.PF_KERNEL_BATCHED, stats=True)
    hist1 = its_histogram(dev.a["newton_its"])
    order = torch.argsort(dev.a["newton_its"].to(torch.int64), descending=True)
    pristine = {k: dev.a[k].clone() for k in MUTABLE if k in dev.a}  # S1, the timed step's input
    # one instrumented run of the timed step: iteration statistics for the flop count
    stats = eng.rstep(dev, dt, kernel=abi.PF_KERNEL_BATCHED, stats=True)
    its_mean = stats["newton_iterations"] / ncells
    hist = its_histogram(dev.a["newton_its"])
    for k in pristine:
        dev.a[k].copy_(pristine[k])

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        total_ms, kern_ms = time_steps(eng, dev, pristine, dt, abi.PF_KERNEL_BATCHED, args.steps, args.warmup)
    ord_total, ord_kern = time_steps(eng, dev, pristine, dt, abi.PF_KERNEL_BATCHED, max(1, min(args.steps, 3)), 1,
                                     order=order)
    if dist:
        # replicas: the slowest rank's time, and the reference loop's
        # rstep_error MAX / iteration sums over the ranks
        from pfgpu.replicas import max_over_ranks, reduce_step_stats
        total_ms = max_over_ranks(total_ms, device="cuda")
        stats = reduce_step_stats(stats, device="cuda")
    value = world * ncells * args.steps / (total_ms * 1e-3)
    kern_avg = float(np.mean(kern_ms))

    # adjoint of the timed step
    adjoint = adjoint_measure(eng, dev, pristine, dt, None, nrep, kern_avg)
    adjoint["first_step"] = adjoint1

    # plain one-thread-per-cell form, same inputs
    p_total, p_kern = time_steps(eng, dev, pristine, dt, abi.PF_KERNEL_PLAIN, max(1, min(args.steps, 3)), 1)
    plain_value = ncells * len(p_kern) / (p_total * 1e-3)

    # roofline: FP64 pipe.  achieved = the reference algorithm's flops per
    # Newton iteration (flops.per_iteration) x the step's Newton iterations /
    # kernel time; also on the kernel's own algorithm (flops.kernel_per_
    # iteration: LDL^T, no scaling) and against the DFMA issue rate ncu states
    # for this part (2 DFMA per SM per clock) at the clock sampled during the
    # timed region
    f_it, tr_it = flops.per_iteration(net)
    k_it, _ = flops.kernel_per_iteration(net)
    flops_per_launch = f_it * its_mean * ncells
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    probe_clocks = {}
    peak = fp64_peak(abi.load(), sms, probe_clocks)
    achieved = flops_per_launch / (kern_avg * 1e-3) / 1e12
    achieved_own = k_it * its_mean * ncells / (kern_avg * 1e-3) / 1e12
    clocks = clk.summary()
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    dfma_peak = 2 * 2 * sms * sm_mhz * 1e6 / 1e12
    state_bytes = sum(v.numel() * v.element_size() for v in dev.a.values())
    # DRAM bytes per cell-solve of the launched kernel measured by ncu on the
    # same workload at 200,000 cells, scaled to this launch:
    #   one lane per cell  profiles/rstep_batched_kernel_n12_200k.txt   6.431 + 4.639 GB
    #   group of lanes     profiles/rstep_group_kernel_g4_n12_200k.txt  0.2232 + 0.1005 GB
    #                      (the second step, queue in cell order)
    grp = eng.launch_config()["lanes_per_cell"] > 1
    per_launch_200k = (0.2232e9 + 0.1005e9) if grp else (6.431e9 + 4.639e9)
    traffic = per_launch_200k / 200_000 * ncells if args.config == "c2" else None
    roofline = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak if peak else None, "traffic": traffic,
                "traffic_unit": "bytes per launch (ncu, scaled by cells)",
                "peak_source": "FP64 DFMA probe (pf_bench_fp64_fma) measured in this run",
                "flops_per_cell_solve": f_it * its_mean, "transcendentals_per_cell_solve": tr_it * its_mean,
                "own_algorithm": {"flops_per_cell_solve": k_it * its_mean, "achieved": achieved_own,
                                  "frac": achieved_own / peak if peak else None},
                "dfma_issue_peak": {"tflops": dfma_peak, "sm_mhz": sm_mhz,
                                    "frac": achieved / dfma_peak, "frac_own_algorithm": achieved_own / dfma_peak,
                                    "probe_frac": peak / dfma_peak,
                                    # the probe against the issue rate at the clock it ran at
                                    "probe_clocks": probe_clocks or None,
                                    "probe_frac_at_its_clock": (
                                        peak / (2 * 2 * sms * probe_clocks["sm_mhz"] * 1e6 / 1e12)
                                        if probe_clocks.get("sm_mhz") else None)},
                "hbm_gbs": state_bytes * 2 / (kern_avg * 1e-3) / 1e9}

    e2e = None
    if not args.no_e2e:
        host = dev.numpy()
        pin = {}
        for k, v in dev.a.items():
            pin[k] = torch.empty(v.shape, dtype=v.dtype, pin_memory=True)
        from pfgpu.network import CellState
        hs = CellState(net, {k: pin[k].numpy() for k in pin})
        h2d = sum(pin[k].numel() * pin[k].element_size() for k in pin if k not in ("mnrl_rate", "status",
                                                                                  "newton_its", "num_substeps"))
        d2h = sum(pin[k].numel() * pin[k].element_size() for k in pin
                  if k in ("total", "pri_molal", "pri_act_coef", "sec_act_coef", "sec_molal", "mnrl_volfrac",
                           "mnrl_rate", "status", "newton_its", "num_substeps"))
        src = {k: pristine[k].cpu().numpy() if k in pristine else host.a[k] for k in pin}
        times = []
        for k in range(args.warmup + args.steps):
            for f in pin:
                np.copyto(hs.a[f], src[f])
            t = time.perf_counter()
            eng.rstep_host(hs, dt)
            el = time.perf_counter() - t
            if k >= args.warmup:
                times.append(el)
        e2e = {"value": ncells * len(times) / sum(times), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}

    constraint = None
    if args.config == "c2":
        constraint = constraint_measure(net, eng, inputs, cpu=(rank == 0 and not args.no_cpu))
        log("constraint:", json.dumps(constraint))

    girt = None
    if not args.no_girt and args.config == "c2":
        for k in pristine:
            dev.a[k].copy_(pristine[k])
        girt = girt_measure(net, eng, dev, max(3, args.steps), max(3, args.warmup), cpu=(rank == 0 and not args.no_cpu))
        log("girt:", json.dumps(girt))

    transport = None
    if not args.no_girt and args.config == "c2":
        for k in pristine:
            dev.a[k].copy_(pristine[k])
        transport = transport_measure(net, dev, max(3, args.steps), max(2, min(args.warmup, 3)),
                                      cpu=(rank == 0 and not args.no_cpu))
        log("transport:", json.dumps(transport))

    cpu = None
    if rank == 0 and not args.no_cpu:
        host = dev.numpy()
        for k in pristine:
            host.a[k] = pristine[k].cpu().numpy()
        cpu = cpu_baseline(net, host, dt)

    hetero = None
    if args.config == "c2" and not args.no_c3:
        host = None
        for k in list(dev.a):
            dev.a[k] = None
        dev = None
        torch.cuda.empty_cache()
        hetero = c3_measure(args, per=args.c3_cells or 500_000, nsteps=args.graph_steps, replays=1,
                            plain=True, eager_steps=0)
        hetero.pop("clocks", None)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": c2_config(cfg, ncells, dt, state_bytes),
                "launch": {"kernel": "batched persistent (PF_KERNEL_BATCHED)", "config": eng.launch_config(),
                           "autotune": tuned,
                           "cell_order": "cell index (natural)"},
                "kernel_ms": kern_avg, "newton_its_per_cell": its_mean,
                "max_newton_its": stats["max_newton_iterations"], "failed_cells": stats["failed_cells"],
                "newton_its_histogram": hist,
                "first_step": {"what": "the first step from the equilibrated state, natural queue order",
                               "value": ncells * len(f1_kern) / (f1_total * 1e-3),
                               "kernel_ms": float(np.mean(f1_kern)),
                               "plain_gpu": {"value": ncells * len(p1_kern) / (p1_total * 1e-3),
                                             "kernel_ms": float(np.mean(p1_kern))},
                               "speedup_vs_plain_gpu": float(np.mean(p1_kern)) / float(np.mean(f1_kern)),
                               "newton_its_per_cell": stats1["newton_iterations"] / ncells,
                               "max_newton_its": stats1["max_newton_iterations"],
                               "failed_cells": stats1["failed_cells"],
                               "newton_its_histogram": hist1},
                "plain_gpu": {"value": plain_value, "kernel_ms": float(np.mean(p_kern))},
                "cost_order": {"what": "the same step, its queue in descending Newton count of the first step",
                               "value": ncells * len(ord_kern) / (ord_total * 1e-3),
                               "kernel_ms": float(np.mean(ord_kern))},
                "speedup_vs_plain_gpu": value / plain_value,
                "adjoint": adjoint, "girt_assembly": girt, "constraint_equilibration": constraint,
                "osrt_transport": transport, "heterogeneous": hetero,
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clocks,
                # per step: the setup pre-pass and the persistent kernel
                "gpu_launches": 2 * args.steps}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
