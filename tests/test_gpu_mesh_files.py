"""GPU: a design read from a gmsh file (jittered tetrahedra, no logical grid:
solves preconditioned by the GPU-built smoothed-aggregation multigrid) with
surface-traction loads, through the OC loop,
against the oracle loop on the same mesh and loads.  Two traction groups
are two load cases (block right-hand side).  Per-iteration compliance 1e-9
relative (FP64) / 1e-6 (mixed), densities 1e-7 / 1e-5.
"""
import numpy as np
import pytest

from oracle import fem as ofem
from oracle import mesh as omesh
from oracle import optim as oopt
from oracle import surface as osurf
from oracle.filters import SpacialFilter as OFilter

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda", 0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tet_mesh_file_oc_loop_matches_oracle(native_lib, tmp_path, precision):
    from sktopt_gb300 import tools
    from sktopt_gb300.core import OC_Config, OC_Optimizer
    from sktopt_gb300.mesh import (LinearElasticity, boundary_facets, create_box_tet,
                                   read_msh, write_msh)
    from sktopt_gb300.mesh import get_points_in_range as rng
    m0 = create_box_tet(8, 4, 4, 2.0, 1.0, 1.0, jitter=0.2, seed=5)
    left = boundary_facets(m0, rng((0, 0), (0, 9), (0, 9)))
    tip = boundary_facets(m0, rng((2.0, 2.0), (0, 9), (0.0, 0.5)))
    top = boundary_facets(m0, rng((1.0, 2.0), (0, 9), (1.0, 1.0)))
    write_msh(tmp_path / "beam.msh", m0,
              boundaries={"dirichlet": left, "neumann_1": tip, "neumann_2": top},
              subdomains={"design": np.arange(m0.nelements)})
    mesh = read_msh(tmp_path / "beam.msh")
    tsk = LinearElasticity.from_mesh_tags(mesh, "all", ["u^3", "u^3"], [-1.0, -0.5], 1.0, 0.3)
    assert tsk.n_tasks == 2 and not mesh.has_grid
    n_iter, radius = 4, 0.35
    cfg = OC_Config(max_iters=n_iter, filter_type="spacial",
                    filter_radius=tools.SchedulerConfig.constant(target_value=radius),
                    p=tools.SchedulerConfig.constant(target_value=3.0),
                    vol_frac=tools.SchedulerConfig.constant(target_value=0.3),
                    move_limit=tools.SchedulerConfig.constant(target_value=0.2),
                    E_min_coeff=1e-9, solver_option="spsolve", precision=precision)
    opt = OC_Optimizer(cfg, tsk, device=_dev())
    opt.parameterize()
    assert opt.fem.engine.amg and opt.fem.engine.multigrid
    # oracle: same mesh, Dirichlet nodes, traction loads and design sets
    om = omesh.GridMesh(mesh.p, mesh.t, "tet", None, None, None)
    loads = osurf.surface_forces(om, [mesh.boundaries["neumann_1"],
                                      mesh.boundaries["neumann_2"]],
                                 ["u^3", "u^3"], [-1.0, -0.5])
    dn = np.nonzero(np.isclose(mesh.p[0], 0.0))[0]
    pb = ofem.ElasticProblem(om, dn, loads)
    design = np.asarray(tsk.design_elements, dtype=np.int64)
    fixed = np.setdiff1d(np.arange(mesh.nelements), design)
    mask = np.zeros(mesh.nelements, bool)
    mask[design] = True
    filt = OFilter(om, radius, mask)
    vol = omesh.elements_volume(om)
    ocfg = oopt.OracleConfig(max_iters=n_iter, p=oopt.Sched("Constant", 3.0, 3.0),
                             vol_frac=oopt.Sched("Constant", 0.3, 0.3),
                             move_limit=oopt.Sched("Constant", 0.2, 0.2),
                             filter_radius=oopt.Sched("Constant", radius, radius),
                             E_min_coeff=1e-9)
    ref = oopt.OracleOptimizer(ocfg, pb, filt, design, fixed, vol)
    ctol, rtol = (1e-9, 1e-7) if precision == "fp64" else (1e-6, 1e-5)
    for k in range(n_iter):
        opt.optimize_steps(1)
        c_ref = ref.step()
        c = opt.recorder.histories["compliance"][-1]
        assert abs(c - c_ref) <= ctol * abs(c_ref), (k, c, c_ref)
        np.testing.assert_allclose(opt._state.rho.cpu().numpy(), ref.rho, rtol=0, atol=rtol)
