"""The SCIP propagator plugin, built and run inside SCIP itself (compiled from the reference sources into
oracle/_ref).  On a machine without an sm_103 GPU the plugin must register, extract exactly the problem's rows,
disable itself with a warning and leave SCIP's own propagation to produce the root fixpoint.  Skipped where the
SCIP build is absent."""
import os
import subprocess

import numpy as np

import pytest

from scip_gb300 import instances
from scip_gb300.build import LIBDIR, build_libgbp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref")
LIBSCIP = os.path.join(REF, "libscip.a")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="module")
def driver(tmp_path_factory, oracle_mod):
    if not os.path.exists(LIBSCIP):
        pytest.skip("SCIP build (oracle/_ref) not present")
    if not oracle_mod.REFDIR or not os.path.exists(os.path.join(oracle_mod.REFDIR, "src", "scip", "scip.h")):
        pytest.skip("SCIP headers not present (REFDIR names the SCIP source tree)")
    build_libgbp()
    out = tmp_path_factory.mktemp("plugin")
    exe = str(out / "plugin_driver")
    src = [os.path.join(ROOT, "tests", "plugin", "plugin_driver.c"),
           os.path.join(ROOT, "scip_gb300", "plugin", "prop_gpulinear.c"),
           os.path.join(ROOT, "scip_gb300", "plugin", "gpulinear_reason.c")]
    inc = ["-I" + os.path.join(REF, "include"), "-I" + os.path.join(oracle_mod.REFDIR, "src"),
           "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "scip_gb300", "plugin")]
    cmd = ["gcc", "-std=c99", "-O1", "-D_XOPEN_SOURCE=600", *inc, "-o", exe, *src, LIBSCIP,
           "-L" + LIBDIR, "-lgbp", "-Wl,-rpath," + LIBDIR, "-lstdc++", "-lm", "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def run(driver, inst, tmp_path, *args):
    p = str(tmp_path / "inst.bin")
    inst.write(p)
    r = subprocess.run([driver, p, *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = dict(l.split(" ", 1) for l in r.stdout.strip().splitlines())
    return lines, r.stdout + r.stderr


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour without a GPU")
def test_plugin_without_gpu_extracts_rows_and_steps_aside(driver, oracle_mod, tmp_path):
    inst = instances.root_mip(0)
    lines, text = run(driver, inst, tmp_path)
    assert lines["active"] == "0"
    assert "propagator <gpulinear> disabled" in text
    m, n, nnz, ok = lines["matrix"].split()
    assert (int(m), int(n), int(nnz), ok) == (inst.m, inst.n, inst.nnz, "1")
    # cons_linear still propagates: the root equals SCIP's own root fixpoint
    _, slb, sub, _ = oracle_mod.run_scip(inst)
    cut, s_lb, s_ub = lines["root"].split()
    assert cut == "0"
    assert float(s_lb) == pytest.approx(float(slb.sum()), rel=1e-12)
    assert float(s_ub) == pytest.approx(float(sub.sum()), rel=1e-12)


def test_replacelinear_switches_cons_linear_propagation_off(driver, tmp_path):
    inst = instances.root_mip(1, m=200, n=500)
    lines, _ = run(driver, inst, tmp_path, "--replace")
    assert lines["propfreq"] == "-1"


@pytest.fixture(scope="module")
def solve_driver(tmp_path_factory, oracle_mod):
    """tests/plugin/solve_driver.c with the plugin on top of the oracle test double (tests/plugin/gbp_oracle_shim.c):
    the plugin's SCIP side -- change log write-back, conflict analysis of cutoffs, reasons -- runs inside SCIP."""
    if not os.path.exists(LIBSCIP):
        pytest.skip("SCIP build (oracle/_ref) not present")
    if not oracle_mod.REFDIR or not os.path.exists(os.path.join(oracle_mod.REFDIR, "src", "scip", "scip.h")):
        pytest.skip("SCIP headers not present (REFDIR names the SCIP source tree)")
    out = tmp_path_factory.mktemp("solve")
    exe = str(out / "solve_driver")
    src = [os.path.join(ROOT, "tests", "plugin", "solve_driver.c"),
           os.path.join(ROOT, "scip_gb300", "plugin", "prop_gpulinear.c"),
           os.path.join(ROOT, "scip_gb300", "plugin", "gpulinear_reason.c"),
           os.path.join(ROOT, "tests", "plugin", "gbp_oracle_shim.c"),
           os.path.join(ROOT, "oracle", "linprop_oracle.c"),
           os.path.join(ROOT, "oracle", "linprop_seq.c")]
    inc = ["-I" + os.path.join(REF, "include"), "-I" + os.path.join(oracle_mod.REFDIR, "src"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "scip_gb300", "plugin"),
           "-I" + os.path.join(ROOT, "oracle")]
    cmd = ["gcc", "-std=c99", "-O1", "-D_XOPEN_SOURCE=600", "-ffp-contract=off", *inc, "-o", exe, *src, LIBSCIP,
           "-lstdc++", "-lm", "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def _solve(exe, path, mode, ranged=False, presolve=False):
    flags = (["ranged"] if ranged else []) + (["presolve"] if presolve else [])
    r = subprocess.run([exe, path, mode, "200000"] + flags, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return dict(l.split(" ", 1) for l in r.stdout.strip().splitlines() if " " in l)


@pytest.mark.parametrize("name", ["enigma", "flugpl", "misc03"])
def test_plugin_replaces_linear_propagation_in_search(solve_driver, oracle_mod, name):
    """SCIP searches (propagation and conflict analysis, no LP) once with cons_linear's propagation and once with the
    gpulinear propagator in its place: both prove the same optimum; every reason SCIP asks the plugin for is
    explained with a row, and the plugin's cutoffs feed conflict analysis."""
    path = os.path.join(oracle_mod.REFDIR, "check", "instances", "MIP", name + ".mps")
    if not os.path.exists(path):
        pytest.skip(f"{name}.mps not shipped")
    plain = _solve(solve_driver, path, "plain")
    gpu = _solve(solve_driver, path, "gpulinear")
    assert plain["status"] == "optimal" and gpu["status"] == "optimal"
    assert float(plain["obj"]) == float(gpu["obj"])
    calls, chg, cut, analysed, asked, resolved, _, active = gpu["gpulinear"].split()
    assert active == "1" and int(calls) > 0 and int(chg) > 0
    assert asked == resolved
    if name != "flugpl":  # flugpl is solved without any conflict
        assert int(resolved) > 0 and int(analysed) > 0 and int(gpu["conflicts"]) > 0


@pytest.mark.parametrize("seed", [5, 6, 7])
def test_plugin_ranged_rows_in_search(solve_driver, tmp_path, seed):
    """Ranged-row propagation on (without artificial constraints) on rows whose integer part shares a divisor: SCIP
    with cons_linear and SCIP with the plugin prove the same optimum, and the plugin explains the changes and
    cutoffs of its ranged rows to conflict analysis with the rows it recorded (gbp_get_ranged_log)."""
    from scip_gb300 import instances, mps
    # no continuous columns: the search has no LP solver for them (LP solver none)
    inst = instances.gcd_rows(np.random.default_rng(seed), 30, 80, equations=True, continuous=False)
    path = str(tmp_path / "gcd.mps")
    mps.write_mps(inst, path, obj=np.random.default_rng(seed + 100).integers(-5, 6, inst.n))
    plain = _solve(solve_driver, path, "plain", ranged=True)
    gpu = _solve(solve_driver, path, "gpulinear", ranged=True)
    assert plain["status"] == gpu["status"] and plain["status"] in ("optimal", "infeasible")
    if plain["status"] == "optimal":
        assert float(plain["obj"]) == float(gpu["obj"])
    calls, chg, cut, analysed, asked, resolved, _, active = gpu["gpulinear"].split()
    assert active == "1" and int(calls) > 0
    assert asked == resolved
    assert int(gpu["rangedreasons"]) > 0


@pytest.mark.parametrize("name", ["enigma", "flugpl", "misc03"])
def test_plugin_replaces_the_specialised_handlers_after_presolving(solve_driver, oracle_mod, name):
    """SCIP's presolving on: linear rows are upgraded to setppc, logicor, knapsack and varbound constraints.  The
    plugin reads their rows (over active variables: negated, aggregated and fixed variables resolved) and, with
    replacespecialised, replaces those handlers' propagation as well as cons_linear's.  Both searches prove the same
    optimum, and every reason SCIP asks for is explained."""
    path = os.path.join(oracle_mod.REFDIR, "check", "instances", "MIP", name + ".mps")
    if not os.path.exists(path):
        pytest.skip(f"{name}.mps not shipped")
    plain = _solve(solve_driver, path, "plain", presolve=True)
    gpu = _solve(solve_driver, path, "gpulinear", presolve=True)
    assert plain["status"] == "optimal" and gpu["status"] == "optimal"
    assert float(plain["obj"]) == float(gpu["obj"])
    calls, chg, cut, analysed, asked, resolved, _, active = gpu["gpulinear"].split()
    assert active == "1" and int(calls) > 0 and int(chg) > 0
    assert asked == resolved


@pytest.fixture(scope="module")
def nodes_driver(tmp_path_factory, oracle_mod):
    """tests/plugin/nodes_driver.c: the plugin's batched entry (SCIPpropagateGpulinearNodes) inside SCIP, on the
    oracle test double, against SCIP's own probing."""
    if not os.path.exists(LIBSCIP):
        pytest.skip("SCIP build (oracle/_ref) not present")
    if not oracle_mod.REFDIR or not os.path.exists(os.path.join(oracle_mod.REFDIR, "src", "scip", "scip.h")):
        pytest.skip("SCIP headers not present (REFDIR names the SCIP source tree)")
    out = tmp_path_factory.mktemp("nodes")
    exe = str(out / "nodes_driver")
    src = [os.path.join(ROOT, "tests", "plugin", "nodes_driver.c"),
           os.path.join(ROOT, "scip_gb300", "plugin", "prop_gpulinear.c"),
           os.path.join(ROOT, "scip_gb300", "plugin", "gpulinear_reason.c"),
           os.path.join(ROOT, "tests", "plugin", "gbp_oracle_shim.c"),
           os.path.join(ROOT, "oracle", "linprop_oracle.c"),
           os.path.join(ROOT, "oracle", "linprop_seq.c")]
    inc = ["-I" + os.path.join(REF, "include"), "-I" + os.path.join(oracle_mod.REFDIR, "src"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "scip_gb300", "plugin"),
           "-I" + os.path.join(ROOT, "oracle")]
    cmd = ["gcc", "-std=c99", "-O1", "-D_XOPEN_SOURCE=600", "-ffp-contract=off", *inc, "-o", exe, *src, LIBSCIP,
           "-lstdc++", "-lm", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.parametrize("name", ["enigma", "flugpl", "lseu", "misc03", "p0548"])
def test_batched_plugin_entry_agrees_with_scip_probing(nodes_driver, oracle_mod, name):
    """SCIPpropagateGpulinearNodes propagates 200 nodes of integer fixings in one call on top of the root's local
    bounds; SCIP then propagates each of them through SCIPpropagateProbing with cons_linear's propagation: the same
    cutoff verdicts and the same integer bounds on every node."""
    path = os.path.join(oracle_mod.REFDIR, "check", "instances", "MIP", name + ".mps")
    if not os.path.exists(path):
        pytest.skip(f"{name}.mps not shipped")
    r = subprocess.run([nodes_driver, path, "200"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [l for l in r.stdout.splitlines() if l.startswith("nodes ")]
    assert line, r.stdout
    f = line[0].split()
    got = {f[i]: f[i + 1] for i in range(len(f) - 1) if not f[i].lstrip("-").isdigit()}
    assert got["success"] == "1"
    assert got["cutoffmismatch"] == "0" and got["intmismatch"] == "0", line[0]
    assert int(got["moved"]) > 0


@pytest.mark.parametrize("rule", ["res", "easy"])
@pytest.mark.parametrize("name", ["bell5", "blend2", "dcmulti", "egout", "enigma", "flugpl", "gt2", "lseu", "misc03",
                                  "p0548", "rgn"])
def test_batched_plugin_entry_in_scip_order_agrees_with_scip_probing(nodes_driver, oracle_mod, name, rule):
    """propagating/gpulinear/sciporder: the batched entry reads the rows again in the order SCIP holds them and
    propagates 200 nodes in SCIP's own order; SCIP propagates each node in probing with no row marked at its start:
    the same cutoff verdicts and integer bounds on every node, continuous bounds within 1e-9 relative or feastol.
    Every MIPLIB instance the reference ships (but semicon1), the residual rule and SCIP's default rule choice."""
    path = os.path.join(oracle_mod.REFDIR, "check", "instances", "MIP", name + ".mps")
    if not os.path.exists(path):
        pytest.skip(f"{name}.mps not shipped")
    args = [nodes_driver, path, "200", "sciporder"] + (["easy"] if rule == "easy" else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [l for l in r.stdout.splitlines() if l.startswith("nodes ")]
    assert line, r.stdout + r.stderr[-2000:]
    f = line[0].split()
    got = {f[i]: f[i + 1] for i in range(len(f) - 1) if not f[i].lstrip("-").isdigit()}
    assert got["success"] == "1", r.stderr[-2000:]
    assert got["cutoffmismatch"] == "0" and got["intmismatch"] == "0" and got["contmismatch"] == "0", \
        line[0] + "\n" + r.stderr[-1500:]


@pytest.mark.parametrize("rule", ["res", "easy"])
@pytest.mark.parametrize("name", ["bell5", "blend2", "dcmulti", "egout", "enigma", "flugpl", "gt2", "lseu", "misc03",
                                  "p0548", "rgn"])
def test_batched_plugin_entry_in_scip_order_after_presolving(nodes_driver, oracle_mod, name, rule):
    """SCIP presolves first (its rows stay linear).  Presolving leaves rows in index order with their tightening
    already done, so SCIP's root does not sort them; the first visit in a node does.  The batched entry uploads such
    rows in the order that visit gives them, and its 200 nodes in SCIP's order equal SCIP's probing."""
    path = os.path.join(oracle_mod.REFDIR, "check", "instances", "MIP", name + ".mps")
    if not os.path.exists(path):
        pytest.skip(f"{name}.mps not shipped")
    r = subprocess.run([nodes_driver, path, "200", "sciporder", rule, "plain", "0", "presolve"], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [l for l in r.stdout.splitlines() if l.startswith("nodes ")][0]
    f = line.split()
    got = {f[i]: f[i + 1] for i in range(len(f) - 1) if not f[i].lstrip("-").isdigit()}
    assert got["success"] == "1", r.stderr[-2000:]
    assert got["cutoffmismatch"] == "0" and got["intmismatch"] == "0" and got["contmismatch"] == "0", \
        line + "\n" + r.stderr[-1500:]


@pytest.mark.parametrize("presolve", ["0", "presolve"])
@pytest.mark.parametrize("name", ["bell5", "blend2", "dcmulti", "egout", "enigma", "flugpl", "gt2", "lseu", "misc03",
                                  "p0548", "rgn"])
def test_batched_plugin_entry_in_scip_order_without_sortvars(nodes_driver, oracle_mod, name, presolve):
    """constraints/linear/sortvars = FALSE: SCIP visits every row in the order presolving left it, and so does the
    batched entry; its 200 nodes in SCIP's order equal SCIP's probing, with and without presolving."""
    path = os.path.join(oracle_mod.REFDIR, "check", "instances", "MIP", name + ".mps")
    if not os.path.exists(path):
        pytest.skip(f"{name}.mps not shipped")
    r = subprocess.run([nodes_driver, path, "200", "sciporder", "res", "nosort", "0", presolve], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [l for l in r.stdout.splitlines() if l.startswith("nodes ")][0]
    f = line.split()
    got = {f[i]: f[i + 1] for i in range(len(f) - 1) if not f[i].lstrip("-").isdigit()}
    assert got["success"] == "1", r.stderr[-2000:]
    assert got["cutoffmismatch"] == "0" and got["intmismatch"] == "0" and got["contmismatch"] == "0", \
        line + "\n" + r.stderr[-1500:]


@pytest.mark.parametrize("rule", ["res", "easy"])
@pytest.mark.parametrize("name", ["bell5", "blend2", "dcmulti", "egout", "enigma", "flugpl", "gt2", "lseu", "misc03",
                                  "p0548", "rgn"])
def test_batched_plugin_entry_below_the_root(nodes_driver, oracle_mod, name, rule):
    """The batched entry at the first search node of depth 3: the nodes' base is that node's local bounds, tighter
    than SCIP's global ones (the binary test reads the global domain).  In SCIP's order the 200 nodes equal SCIP's
    probing from that node; in rounds the cutoff verdicts and integer bounds do."""
    path = os.path.join(oracle_mod.REFDIR, "check", "instances", "MIP", name + ".mps")
    if not os.path.exists(path):
        pytest.skip(f"{name}.mps not shipped")
    for mode in ("sciporder", "rounds"):
        r = subprocess.run([nodes_driver, path, "200", mode, rule, "plain", "3"], capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        line = [l for l in r.stdout.splitlines() if l.startswith("nodes ")][0]
        f = line.split()
        got = {f[i]: f[i + 1] for i in range(len(f) - 1) if not f[i].lstrip("-").isdigit()}
        assert got["success"] == "1", r.stderr[-2000:]
        assert got["cutoffmismatch"] == "0" and got["intmismatch"] == "0", line
        if mode == "sciporder":
            assert got["contmismatch"] == "0", line + "\n" + r.stderr[-1500:]


@pytest.mark.parametrize("rule", ["res", "easy"])
@pytest.mark.parametrize("seed", [5, 6, 7, 8])
def test_batched_plugin_entry_with_ranged_rows(nodes_driver, tmp_path, seed, rule):
    """Ranged-row propagation on, on rows whose integer part shares a divisor: SCIP's probing keeps every row's
    rangedrowpropagated mark, so its nodes run no ranged-row rule, and neither does the batched entry.  In SCIP's
    order the 200 nodes equal SCIP's probing (cutoff verdicts, integer bounds, continuous bounds within tolerance);
    in rounds the cutoff verdicts do (the rounds reach other fixpoints on at most a few integer bounds)."""
    from scip_gb300 import instances, mps
    inst = instances.gcd_rows(np.random.default_rng(seed), 300, 900, equations=True, continuous=False)
    path = str(tmp_path / f"gcd{seed}.mps")
    mps.write_mps(inst, path, obj=np.random.default_rng(seed + 100).integers(-5, 6, inst.n))
    for mode in ("sciporder", "rounds"):
        r = subprocess.run([nodes_driver, path, "200", mode, rule, "ranged"], capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        line = [l for l in r.stdout.splitlines() if l.startswith("nodes ")][0]
        f = line.split()
        got = {f[i]: f[i + 1] for i in range(len(f) - 1) if not f[i].lstrip("-").isdigit()}
        assert got["success"] == "1" and got["cutoffmismatch"] == "0", line
        if mode == "sciporder":
            assert got["intmismatch"] == "0" and got["contmismatch"] == "0", line + "\n" + r.stderr[-1500:]
        else:
            assert int(got["intmismatch"]) <= 2, line


def test_constraint_with_a_fixed_variable_added_while_solving(tmp_path, oracle_mod):
    """SCIP's own scenario tests/src/cons/linear/fixedvar.c with the propagator in place: after bell5's root a
    variable fixed to 0 and a linear constraint over it and five more variables are added, and the search continues
    to node 5 with cons_linear's propagation delayed to depth 3.  The propagator takes up the new row (one more row;
    the fixed variable becomes a constant) and keeps running."""
    if not os.path.exists(LIBSCIP):
        pytest.skip("SCIP build (oracle/_ref) not present")
    if not oracle_mod.REFDIR or not os.path.exists(os.path.join(oracle_mod.REFDIR, "src", "scip", "scip.h")):
        pytest.skip("SCIP headers not present (REFDIR names the SCIP source tree)")
    path = os.path.join(oracle_mod.REFDIR, "check", "instances", "MIP", "bell5.mps")
    if not os.path.exists(path):
        pytest.skip("bell5.mps not shipped")
    exe = str(tmp_path / "fixedvar_driver")
    src = [os.path.join(ROOT, "tests", "plugin", "fixedvar_driver.c"),
           os.path.join(ROOT, "scip_gb300", "plugin", "prop_gpulinear.c"),
           os.path.join(ROOT, "scip_gb300", "plugin", "gpulinear_reason.c"),
           os.path.join(ROOT, "tests", "plugin", "gbp_oracle_shim.c"),
           os.path.join(ROOT, "oracle", "linprop_oracle.c"),
           os.path.join(ROOT, "oracle", "linprop_seq.c")]
    inc = ["-I" + os.path.join(REF, "include"), "-I" + os.path.join(oracle_mod.REFDIR, "src"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "scip_gb300", "plugin"),
           "-I" + os.path.join(ROOT, "oracle")]
    subprocess.run(["gcc", "-std=c99", "-O1", "-D_XOPEN_SOURCE=600", "-ffp-contract=off", *inc, "-o", exe, *src,
                    LIBSCIP, "-lstdc++", "-lm", "-lpthread"], check=True, capture_output=True)
    r = subprocess.run([exe, path], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    f = r.stdout.split()
    got = {f[i]: f[i + 1:i + 3] for i in range(len(f)) if f[i] in ("rows", "nnz", "active", "calls", "status")}
    before, after = int(got["rows"][0]), int(got["rows"][1])
    assert before > 0 and after == before + 1
    assert got["active"][0] == "1" and int(got["calls"][0]) > 0

