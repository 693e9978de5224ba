"""The reaction half of the operator-split time loop, captured in a CUDA graph.

One operator-split time step of PFLOTRAN's OSRT mode does, for the cells
(`pm_osrt.F90:115-153`, `pmc_subsurface_osrt.F90:276-386`):

    RTUpdateAuxVars(cells, act coefs = F)        totals from pri_molal
    RTUpdateActivityCoefficients                 when the frequency is TIMESTEP
    transport solve of the totals                optional (TransportStage,
                                                 pmc_subsurface_osrt.F90:259-330)
    RStep in every cell                          the reaction step

`OperatorSplitLoop` runs that sequence for one or more reaction networks
(each with its own engine and cell state, as when a domain holds several
chemical systems), with the batched kernel's work queue ordered by the
previous step's Newton counts (longest cells first).  `capture(nsteps)`
records `nsteps` consecutive steps of every network into one CUDA graph;
`replay()` launches it.  Nothing in a step synchronises with the host (the
transport solve runs a fixed schedule, pf_transport_enqueue), so the graph
holds the whole time loop; the per-cell status and iteration arrays and the
transport solver's counters carry the results out.
"""
from __future__ import annotations

from dataclasses import dataclass

from . import abi


@dataclass
class TransportStage:
    """The transport solve of a member's totals before its reaction step: a
    pfgpu.transport.OSTransport on the member's grid and a fixed schedule
    (OSTransport.schedule() of an adaptive step gives one)."""
    solver: object
    inner_iterations: int
    refinements: int
    rtol: float = 1e-10


class OperatorSplitLoop:
    def __init__(self, members, dt: float = 0.0, kernel: int = abi.PF_KERNEL_BATCHED, cost_order: bool = True,
                 concurrent: bool = False, multi: bool = False):
        """members: sequence of (ReactionEngine, CellState on the device) or
        (ReactionEngine, CellState, TransportStage).
        dt: uniform step [s]; ignored by the reaction step of states that
        carry a per-cell dt; a member with transport needs dt > 0.
        cost_order: each step's work queue takes the cells in descending
        Newton count of the previous step (stiffest first).  It pays where
        the counts have a long tail (a heterogeneous mix with counts in the
        hundreds: 22.2 s against 25.7 s for 50 steps of eight networks);
        where every cell takes a few iterations, cell order is about 2 %
        faster (neighbouring cells share memory sectors), so pass False.
        concurrent: run each member's step on its own stream (forked from
        and joined back into the calling stream every step), so that one
        network's queue tail overlaps the next network's work.
        multi: the reaction steps of all members in one persistent launch
        (pf_rstep_multi, members in the given order: list the costliest
        first), after every member's auxvar update and transport."""
        self.members = [tuple(m) if len(m) == 3 else (m[0], m[1], None) for m in members]
        self.dt = float(dt)
        for _, st, tr in self.members:
            if not self.dt > 0.0 and (st.a.get("dt_cell") is None or tr is not None):
                raise ValueError("dt must be > 0 for states without a per-cell dt and for transport")
        self.kernel = kernel
        self.cost_order = cost_order
        self.graph = None
        self.nsteps = 0
        self.concurrent = concurrent
        self.multi = multi
        if multi and (concurrent or kernel != abi.PF_KERNEL_BATCHED):
            raise ValueError("multi runs the batched kernel on the calling stream")
        self._streams = None

    def _order(self, st):
        import torch
        if not self.cost_order or self.kernel != abi.PF_KERNEL_BATCHED:
            return None
        return torch.argsort(st.a["newton_its"].to(torch.int64), descending=True)

    def _member_step(self, eng, st, tr, react=True):
        eng.update_auxvars(st, False)
        if eng.net.options["act_coef_update_frequency"] == abi.PF_ACT_COEF_TIMESTEP:
            eng.update_activity_coefs(st)
        if tr is not None:
            tr.solver.enqueue(st, self.dt, tr.inner_iterations, tr.refinements, tr.rtol)
        if react:
            # a state's per-cell dt array, when present, overrides dt
            dt = self.dt if self.dt > 0.0 else 1.0
            eng.rstep(st, dt, kernel=self.kernel, stats=False, order=self._order(st))

    def step(self):
        """One operator-split reaction step of every member, enqueued on the
        current stream (and, when concurrent, on per-member streams joined
        back into it); no host synchronisation."""
        import torch
        if self.multi:
            from .engine import rstep_multi
            orders = [self._order(st) for _, st, _ in self.members]
            for eng, st, tr in self.members:
                self._member_step(eng, st, tr, react=False)
            rstep_multi([(eng, st) for eng, st, _ in self.members], self.dt if self.dt > 0.0 else 1.0,
                        stats=False, orders=orders)
            return
        if not self.concurrent:
            for eng, st, tr in self.members:
                self._member_step(eng, st, tr)
            return
        main = torch.cuda.current_stream()
        if self._streams is None:
            self._streams = [torch.cuda.Stream() for _ in self.members]
        fork = torch.cuda.Event()
        fork.record(main)
        joins = []
        for (eng, st, tr), s in zip(self.members, self._streams):
            s.wait_event(fork)
            with torch.cuda.stream(s):
                self._member_step(eng, st, tr)
                ev = torch.cuda.Event()
                ev.record(s)
                joins.append(ev)
        for ev in joins:
            main.wait_event(ev)

    def capture(self, nsteps: int):
        """Record nsteps steps into one CUDA graph.  Scratch is reserved
        first, so nothing allocates inside the capture; run at least one step
        eagerly before capturing (lazy initialisation of the sort and of the
        kernels' launch attributes).  Capturing enqueues no work: the state
        is unchanged until replay()."""
        import torch
        for eng, st, _ in self.members:
            eng.reserve(st.ncells)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for _ in range(nsteps):
                self.step()
        self.graph, self.nsteps = g, nsteps
        return g

    def replay(self):
        if self.graph is None:
            raise RuntimeError("capture() first")
        self.graph.replay()

    def summary(self):
        """Host reduction of the per-cell outputs of the last step (the
        reference's rstep_error MAX and iteration sums)."""
        out = []
        for eng, st, tr in self.members:
            its = st.a["newton_its"]
            row = dict(ncomp=eng.net.ncomp, cells=st.ncells, failed_cells=int((st.a["status"] != 0).sum()),
                       newton_iterations=int(its.sum()), max_newton_iterations=int(its.max()),
                       max_substeps=int(st.a["num_substeps"].max()))
            if tr is not None:
                row["transport"] = tr.solver.read_stats(tr.rtol)
            out.append(row)
        return out
