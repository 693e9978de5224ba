"""Algorithmic FP64 work of the reference's RReact iteration.

Counts the floating-point operations the reference performs per Newton
iteration (src/pflotran/reaction.F90 RReact :3851-4045 with RTotalAqueous
:4665-4759, RTAccumulation[Derivative] :5710-5848, RKineticMineral
reaction_mineral.F90:647-1078 without prefactors, RSolve :5457-5516 and the
Crout LU utility.F90:597-735): add/sub/mul/div each 1, a fused multiply-add 2,
sqrt 1.  exp/log/pow calls are counted separately as transcendentals.
These are the units of the FP64 roofline ("algorithmic flops").  The counts
are read off the reference's loops (one term per statement, in the order of
the routines named above); tests/test_flops.py checks them against the same
arithmetic counted op by op in a run of the oracle built with a counting
scalar (within a few per cent, never above it).
"""
from __future__ import annotations


def per_iteration(net, mineral_active=None):
    """(flops, transcendentals) of one RReact Newton iteration that goes on
    to the solve and update (the common case)."""
    n = net.ncomp
    s = [int(net.sec_nspec[i]) for i in range(net.nsec)]
    t = [int(net.mnrl_nspec[m]) for m in range(net.nmnrl)]
    act = mineral_active if mineral_active is not None else [True] * len(t)
    f = 0
    tr = 0
    # RTotalAqueous
    tr += 2 * n
    f += n
    for si in s:
        f += 1 + 2 * si + 1 + 2 * si + si * 3 + 2 * si * si
        tr += 1 + si
    f += n + n * n
    # RTAccumulation, derivative, residual
    f += 3 + n + 4 + n * n + 2 * n
    # RKineticMineral
    tr += 2 * n
    f += n
    for ti, a in zip(t, act):
        f += 1 + 2 * ti + 1
        tr += 1
        if a:
            f += 1 + 3 + 2 + 2 * ti + 1 + 4 * ti + 3 * ti * ti
            tr += ti
    # norms and tests
    f += 2 * n + 1 + 1
    # RSolve scaling
    f += n + n + 2 * n * n
    # LU
    f += n
    for j in range(n):
        f += sum(2 * i for i in range(j))
        f += sum(2 * j + 1 for _ in range(j, n))
        f += (n - 1 - j)
    f += n - 1
    # back substitution
    f += sum(2 * i for i in range(n)) + sum(2 * (n - 1 - i) + 1 for i in range(n))
    # update + relative change
    f += 3 * n + 2 * n
    tr += n
    return f, tr


def kernel_per_iteration(net):
    """(flops, transcendentals) of one Newton iteration of the batched step
    kernels as they run (log formulation, LDL^T, csrc/pfgpu_group.cuh and
    pfgpu_batched.cuh), counted from their loops with the same units:
    power table (a, a^2, and 1/a, 1/a^2 for species with a negative
    coefficient), product-form complexes (one multiply per species, no
    exp), the minerals' Q/K and rate law, the residual rows, the lower
    triangle of the symmetric Jacobian entry by entry, LDL^T with the
    forward solve alongside, D^-1, the backward solve, and the update (one
    exp per species).  No row or column scaling and no pivot search: the
    kernel's own algorithm is about half the reference's factorisation
    work, so a roofline on these counts is lower than one on
    per_iteration's."""
    n = net.ncomp
    s = [int(net.sec_nspec[i]) for i in range(net.nsec)]
    t = [int(net.mnrl_nspec[m]) for m in range(net.nmnrl)]
    neg = set()
    for i in range(net.nsec):
        for k in range(s[i]):
            if net.sec_stoich[i, k] < 0:
                neg.add(int(net.sec_spec[i, k]))
    for m in range(net.nmnrl):
        for k in range(t[m]):
            if net.mnrl_stoich[m, k] < 0:
                neg.add(int(net.mnrl_spec[m, k]))
    f = 3                                   # a_acc, b_tot
    f += 2 * n + 2 * len(neg)               # power table
    f += sum(s)                             # complexes: K' prod a^nu
    f += sum(ti + 12 for ti in t)           # minerals: Q/K, affinity, rate, dIm/dlnQ
    f += 2 * sum(s) + n + 3 * n + 4 * n     # rows: sum nu s, a_acc *, totals, residual
    f += 2 * sum(t) + 2 * n                 # mineral residual terms, |r|^2
    f += sum(si * (si + 1) for si in s)     # entries: complexes' nu_i nu_j s
    f += sum(ti * (ti + 1) for ti in t)     # entries: minerals' nu_i nu_j f
    f += n + n * (n + 1) // 2               # diagonal m_i, a_acc * entry
    f += 1 + n                              # norm
    f += n + 3 * n * (n - 1) // 2 + (n - 1) * n * (n + 1) // 3  # LDL^T + forward solve
    f += n + n * (n - 1)                    # D^-1, backward solve
    f += 4 * n                              # update and relative-change test
    return f, n


def girt_per_cell(net, offdiag_blocks: float):
    """FP64 flops (FMA = 2) and transcendental calls per cell of one
    global-implicit assembly (pf_girt_assemble) as its cell kernel computes
    it: the power table, speciation in product form, totals, the packed
    symmetric accumulation of sum_i nu nu s, the kinetic minerals and their
    derivative factors, the diagonal block and `offdiag_blocks` scaled copies
    of d total/d m, and the residual row.  logK(T) of a temperature-dependent
    reaction is 4 terms and two corrected quotients per reaction with ln T
    once per cell, then one exp per reaction; an isothermal network takes K
    from the block's table (no transcendental per cell)."""
    n, ns, nm = net.ncomp, net.nsec, net.nmnrl
    k_s = [int(c) for c in net.sec_nspec]
    k_m = [int(c) for c in net.mnrl_nspec] if nm else []
    neg = set()
    for i, k in enumerate(k_s):
        neg.update(int(net.sec_spec[i, j]) for j in range(k) if net.sec_stoich[i, j] < 0)
    for m, k in enumerate(k_m):
        neg.update(int(net.mnrl_spec[m, j]) for j in range(k) if net.mnrl_stoich[m, j] < 0)
    nn, nsym = n * n, n * (n + 1) // 2
    f = 0
    f += 2 * n + 2 * len(neg)               # a = m gamma, a^2; 1/a, 1/a^2
    f += sum(k + 1 for k in k_s)            # s = K prod a^nu / gamma
    f += sum(2 * k for k in k_s) + n        # totals += nu s, den scaling
    f += sum(k * (k + 1) for k in k_s)      # packed sum_i nu_r nu_c s_i (FMA)
    f += sum(3 * k + 15 for k in k_m)       # QK product, affinity, rate, residual, dIm/dQK QK den
    f += 2 * nsym + n                       # den (E + delta m)
    f += 2 * nn + sum(2 * k * k for k in k_m)  # diagonal block: cdiag e + mineral part
    f += nn * offdiag_blocks                # the scaled copies
    f += n * (3 * 7 + 6)                    # residual row
    temp_dep = not net.options.get("isothermal", 1) and net.sec_logKcoef is not None
    tr = 1 + ns + nm if temp_dep else 0     # ln T, exp per reaction
    if temp_dep:
        f += 12 * (ns + nm)                 # logK(T): 4 terms, two corrected quotients, ln 10 scaling
    return float(f), float(tr)
