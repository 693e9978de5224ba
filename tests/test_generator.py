"""Why the synthetic networks keep the non-H stoichiometry positive.

The benchmark networks are described as integer stoichiometry in {-2..2} at
density 0.3 with log10 K ~ U[-15, 15] and totals log10 U[-6, -2] under a
charge balance on H+.  Drawn that way literally (signed=True), the network
admits no such cells: the TOTAL + charge-balance constraints have no solution
(the oracle's constraint Newton, 200 iterations, finds none), and starting
from free-ion molalities instead every cell holds a complex above 1e20
mol/kg, since a complex with K = 1e15 and a coefficient -2 on a species at
1e-8 mol/kg is 1e31 mol/kg.  pfgpu.generate therefore draws the non-H
coefficients from {1, 2} (H+ keeps {-2, -1, 1, 2}), and these tests hold
both facts and the feasibility of the draw that is used.
"""
import numpy as np
import pytest

from pfgpu import generate
from pfgpu.network import default_options


def _equilibrated(oracle, net, ncells, seed):
    st, ct, cc = generate.random_cells(net, ncells, seed=seed)
    eq = net.with_options(max_relative_change_tolerance=1e-6, max_residual_tolerance=1e-12,
                          max_rel_residual_tolerance=1e-8, maximum_reaction_iterations=200)
    _, its = oracle.equilibrate(eq, st, ct, cc, nthreads=8)
    return float((its > 0).mean())


@pytest.mark.parametrize("seed", [12, 13])
def test_signed_stoichiometry_has_no_feasible_cells(oracle, seed):
    net = generate.random_network(12, 40, 6, seed=seed, signed=True, options=default_options(isothermal=0))
    assert (net.sec_stoich[:, :] < 0).sum() > 20  # the draw is signed
    assert _equilibrated(oracle, net, 200, seed=1212) < 0.01
    # free-ion molalities instead: some complex is far above any solubility
    st, ct, cc = generate.random_cells(net, 500, seed=1212, free=True)
    lm = np.log10(cc)
    ls = np.full((net.nsec, cc.shape[1]), 0.0)
    for i in range(net.nsec):
        ls[i] = -net.sec_logK[i]
        for k in range(net.sec_nspec[i]):
            ls[i] += net.sec_stoich[i, k] * lm[net.sec_spec[i, k]]
    assert ls.max(axis=0).min() > 20.0


def test_positive_stoichiometry_is_feasible(oracle):
    net = generate.random_network(12, 40, 6, seed=12, options=default_options(isothermal=0))
    assert _equilibrated(oracle, net, 200, seed=1212) > 0.95
