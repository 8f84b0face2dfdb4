"""The CUDA path on the golden fixtures, the seeded cases and the MIPLIB instances the reference ships: bit-identical
to the oracle on every fixture instance (root fixpoint through the plain path, nodes through the batched kernel),
hence the same agreement with SCIP's own results that tests/test_golden_cpu.py and tests/test_mps_cpu.py record."""
import numpy as np
import pytest

import golden_cases as G
from scip_gb300 import gbp

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tag", ["res", "easy"])
@pytest.mark.parametrize("case", G.CASES + G.MIPLIB_CASES)
def test_gpu_equals_oracle_on_golden(gpu_prop, oracle_mod, case, tag):
    inst, z = G.load(case)
    maxeasy = 0.0 if tag == "res" else 1e6
    par = oracle_mod.params(maxeasy)
    orc = oracle_mod.Oracle(inst)
    gpu_prop.set_params(gbp.default_params(maxeasy=maxeasy))
    gpu_prop.set_batch_shape(128, 0)
    gpu_prop.upload(inst)
    lb, ub, cut, _ = gpu_prop.propagate(inst.lb, inst.ub)
    olb, oub, ores = orc.propagate(inst.lb, inst.ub, par)
    assert cut == bool(ores.cutoff)
    if not cut:
        assert np.array_equal(lb, olb) and np.array_equal(ub, oub)
    nb = G.nodes_of(z)
    if nb is None:
        return
    rlb, rub = z[f"{tag}_rootlb"], z[f"{tag}_rootub"]
    r = gpu_prop.propagate_nodes(rlb, rub, nb)
    o = orc.propagate_nodes(rlb, rub, nb, par, cap=inst.n)
    assert np.array_equal(r.cutoff, o["cutoff"])
    scip = G.Agreement()
    for k in range(nb.nnodes):
        if r.cutoff[k]:
            scip.add(inst.isint, None, G.scip_node(z, tag, k, rlb, rub))
            continue
        c, l, u = r.node(k)
        n = o["n"][k]
        a, b = np.argsort(c), np.argsort(o["col"][k, :n])
        assert np.array_equal(c[a], o["col"][k, :n][b])
        assert np.array_equal(l[a], o["lb"][k, :n][b]) and np.array_equal(u[a], o["ub"][k, :n][b])
        L, U = rlb.copy(), rub.copy()
        L[c], U[c] = l, u
        scip.add(inst.isint, (L, U), G.scip_node(z, tag, k, rlb, rub))
    assert scip.cutoff_mismatch == 0 and scip.int_exact == scip.problems
