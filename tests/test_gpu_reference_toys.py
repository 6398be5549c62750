"""The reference's own toy problems (sktopt/mesh/toy_problem.py:51-144)
through the flows of its global-flow test (tests/test_global_flow.py:105-150):
``toy_test()`` with ``OC_Config``'s defaults (Helmholtz filter r = 0.01, p and
beta continuation, sawtooth move limit, vf 0.8, Emin 1e-3, direct solves)
and ``toy2()`` (two load cases from mesh tags) with that test's log-MOC
configuration (p Step 1 -> 3 in 3 steps, vf Step with target 0.6), each
for several iterations against the oracle loop on the same mesh.  The
oracle side selects the supports and the loaded facets by brute force over
all element faces and integrates the surface loads with its own rules:
compliance 1e-9 relative, densities 1e-7 (FP64 path).
"""
import numpy as np
import pytest

from oracle import fem as ofem
from oracle import filters as ofilt
from oracle import mesh as omesh
from oracle import optim as oopt
from oracle import surface as osurf

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda", 0)


def _facets_by_midpoint(p, t, box, boundary_only):
    """All element faces, each geometric face once (lowest element first),
    whose midpoint lies in the closed box; as rows (element, local face)."""
    from sktopt_gb300.mesh.grid import element_faces
    faces = element_faces("hex")
    seen, out = {}, []
    count = {}
    for e in range(t.shape[1]):
        for f, loc in enumerate(faces):
            key = tuple(sorted(t[list(loc), e]))
            count[key] = count.get(key, 0) + 1
            if key not in seen:
                seen[key] = (e, f)
    for key, (e, f) in sorted(seen.items(), key=lambda kv: kv[1]):
        if boundary_only and count[key] != 1:
            continue
        mid = p[:, list(key)].mean(axis=1)
        if all(lo <= mid[a] <= hi for a, (lo, hi) in enumerate(box)):
            out.append((e, f))
    return np.array(out, dtype=np.int64).reshape(-1, 2)


def _oracle_problem(tsk, groups, dirs, values, dirichlet_box, boundary_only):
    mesh = tsk.mesh
    om = omesh.GridMesh(mesh.p, mesh.t, "hex", None, None, None)
    p, t = mesh.p, mesh.t
    dfac = _facets_by_midpoint(p, t, dirichlet_box, boundary_only)
    from sktopt_gb300.mesh.grid import facet_nodes_of
    dn = np.unique(facet_nodes_of(mesh, dfac))
    fac = [_facets_by_midpoint(p, t, b, boundary_only) for b in groups]
    loads = osurf.surface_forces(om, fac, dirs, values)
    pb = ofem.ElasticProblem(om, dn, loads, E0=210e3, nu=0.3)
    return om, pb, fac


def _run(opt, ref, n_iter):
    for k in range(n_iter):
        opt.optimize_steps(1)
        c_ref = ref.step()
        c = opt.recorder.histories["compliance"][-1]
        assert abs(c - c_ref) <= 1e-9 * abs(c_ref), (k, c, c_ref)
        np.testing.assert_allclose(opt._state.rho.cpu().numpy(), ref.rho, rtol=0, atol=1e-7)


def _common(tsk, om):
    design = np.asarray(tsk.design_elements, dtype=np.int64)
    fixed = np.setdiff1d(np.arange(tsk.mesh.nelements), design)
    mask = np.zeros(tsk.mesh.nelements, bool)
    mask[design] = True
    vol = omesh.elements_volume(om)
    return design, fixed, mask, vol


def test_toy_test_oc_defaults_matches_oracle(native_lib):
    from sktopt_gb300.core import OC_Config, OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.toy_test()
    assert tsk.mesh.nelements == 8 * 6 * 4
    om, pb, fac = _oracle_problem(
        tsk, [((8.0 - 1.2, 8.1), (2.4, 3.6), (4.0 - 1.2, 4.0))], ["u^3"], [-100.0],
        ((0.0, 0.03), (0.0, 6.0), (0.0, 4.0)), boundary_only=False)
    # the loaded facets include interior ones (scikit-fem's facets_satisfying)
    assert len(fac[0]) == 9
    np.testing.assert_allclose(tsk.neumann_linear[0], pb.forces[0], rtol=0, atol=1e-12)
    n_iter = 4
    cfg = OC_Config(max_iters=n_iter)
    assert cfg.filter_type == "helmholtz"
    opt = OC_Optimizer(cfg, tsk, device=_dev())
    opt.parameterize()
    design, fixed, mask, vol = _common(tsk, om)
    filt = ofilt.HelmholtzFilterNodal(om, vol, 0.01, mask)
    ref = oopt.OracleOptimizer(oopt.OracleConfig(max_iters=n_iter), pb, filt, design, fixed,
                               vol)
    _run(opt, ref, n_iter)


def test_toy2_logmoc_matches_oracle(native_lib):
    from sktopt_gb300 import tools
    from sktopt_gb300.core import LogMOC_Config, LogMOC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.toy2()
    assert tsk.mesh.nelements == 27 * 27 * 4 and tsk.n_tasks == 2
    eps = 0.3
    om, pb, fac = _oracle_problem(
        tsk, [((8.0, 8.0), (8.0 - eps, 8.0), (0.0, 1.0)), ((8.0, 8.0), (0.0, eps), (0.0, 1.0))],
        ["u^2", "u^2"], [-1.0, 1.0], ((0.0, 0.05), (0.0, 8.0), (0.0, 1.0)),
        boundary_only=True)
    for a, b in zip(tsk.neumann_linear, pb.forces):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-14)
    n_iter = 3
    S = tools.SchedulerConfig
    cfg = LogMOC_Config(p=S(init_value=1.0, target_value=3.0, num_steps=3, scheduler_type="Step"),
                        vol_frac=S(target_value=0.6, scheduler_type="Step"), max_iters=n_iter)
    opt = LogMOC_Optimizer(cfg, tsk, device=_dev())
    opt.parameterize()
    design, fixed, mask, vol = _common(tsk, om)
    filt = ofilt.HelmholtzFilterNodal(om, vol, 0.01, mask)
    ocfg = oopt.OracleConfig(method="logmoc", max_iters=n_iter, p=oopt.Sched("Step", 1.0, 3.0, 3),
                             vol_frac=oopt.Sched("Step", None, 0.6, None))
    ref = oopt.OracleOptimizer(ocfg, pb, filt, design, fixed, vol)
    _run(opt, ref, n_iter)
