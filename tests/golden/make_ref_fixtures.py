"""Golden fixtures produced by the reference's own code (scikit-topt 0.3.9).

The reference package imports scikit-fem, numba, PyAMG, matplotlib and meshio
at module level, and none of them is installed here.  This script puts a
permissive stand-in module in front of each missing package (attribute
access returns an inert class, ``numba.njit`` returns the function itself,
``numba.prange`` is ``range``), imports the unmodified reference package from
its source tree, and runs the parts of the hot path that are plain NumPy /
SciPy:

* ``core/projection.py``          Heaviside projection and its derivative
* ``core/derivatives.py``         SIMP / RAMP moduli, dE/drho, dC/drho
* ``fea/composer.py``             SIMP / RAMP interpolation, Lame constants,
                                  hexahedron (6-tet) and tetrahedron volumes
* ``mesh/utils.py``               orientation fixes, get_elements_by_nodes
* ``mesh/task_common.py``         FEMDomain.from_nodes design sets
* ``tools/scheduler.py``          every schedule kind through Schedulers
* ``filters/spacial.py``          the Gaussian filter matrix,
                                  SpacialFilter.forward / gradient
* ``core/optimizers/oc.py``       bisection_with_physical_volume and
                                  OC_Optimizer.rho_update
* ``core/optimizers/logmoc.py``   lagrangian_log_update and
                                  LogMOC_Optimizer.rho_update
* ``core/optimizers/common_density.py``  the driver loop DensityMethod.
                                  _optimize_impl itself, with its FEM plugin
                                  replaced (see below)

What is NOT the reference here: the finite-element arithmetic that the
reference delegates to scikit-fem (element matrices, assembly, ``enforce``,
the strain-energy functional) and the nodal Helmholtz filter (assembled by
scikit-fem).  In the driver-loop fixtures a FEM plugin with the reference's
interface (``objectives_multi_load`` writing ``u_dofs`` in place,
``energy_multi_load``) wraps the NumPy/SciPy restatement in ``oracle/``; the
reference's driver, filter, projection, sensitivity formula, OC / log-MOC
updates, schedules and masks do everything else.  The mesh (skfem's
``MeshHex.init_tensor`` numbering) also comes from ``oracle/mesh.py``.

Two things are changed for speed only, with identical results:
``SpacialFilter.forward`` rebuilds its matrix on every call
(spacial.py:139-149); the loop fixtures reuse the matrix while the radius is
unchanged.  Files the driver exports (VTU, images, progress plots) are not
written.

Run from the repository root (the reference tree must be present):

    python tests/golden/make_ref_fixtures.py [--c1]

``--c1`` also runs the 60x20x20 cantilever for 30 iterations (about half
an hour: one direct solve of 80,703 DOFs per iteration).  Outputs:
tests/golden/ref_*.npz and ref_config_defaults.json.
"""
from __future__ import annotations

import argparse
import importlib.abc
import importlib.machinery
import os
import sys
import tempfile
import time
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = "/root/reference/scikit-topt"
STUBBED = ("skfem", "numba", "pyamg", "matplotlib", "meshio", "pyvista", "petsc4py",
           "imageio")


# --------------------------------------------------------------------------
# stand-ins for the packages that are not installed
def _stand_in(name):
    m = types.ModuleType(name)
    m.__path__ = []

    def getattr_(attr, _m=m):
        if attr.startswith("__"):
            raise AttributeError(attr)
        if attr in ("njit", "jit"):
            def njit(*a, **k):
                if len(a) == 1 and callable(a[0]) and not k:
                    return a[0]
                return lambda f: f
            return njit
        if attr == "prange":
            return range
        cls = type(attr, (), {"__init__": lambda self, *a, **k: None,
                              "__call__": lambda self, *a, **k: None})
        setattr(_m, attr, cls)
        return cls
    m.__getattr__ = getattr_
    return m


class _StandInFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in STUBBED:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        return _stand_in(spec.name)

    def exec_module(self, module):
        pass


def import_reference():
    if not os.path.isdir(REF_SRC):
        raise SystemExit(f"reference source tree not found at {REF_SRC}")
    sys.meta_path.insert(0, _StandInFinder())
    sys.path.insert(0, REF_SRC)
    import logging
    import sktopt  # noqa: F401
    logging.getLogger().setLevel(logging.WARNING)
    return sktopt


sys.path.insert(0, ROOT)
from oracle import fem as ofem          # noqa: E402
from oracle import mesh as omesh        # noqa: E402
from oracle import problems             # noqa: E402


def fake_mesh(sk, m):
    """An instance of the stand-in ``skfem.MeshHex`` / ``MeshTet`` class
    carrying the oracle mesh's p and t (what the reference reads)."""
    import skfem
    cls = skfem.MeshHex if m.t.shape[0] == 8 else skfem.MeshTet
    obj = cls()
    obj.p = np.asarray(m.p, float)
    obj.t = np.asarray(m.t, np.int64)
    obj.nelements = m.t.shape[1]
    obj.nvertices = m.p.shape[1]
    return obj


class FakeBasis:
    """What FEMDomain.from_nodes reads from an skfem vector basis on Hex1:
    ``mesh``, ``N`` and ``get_dofs(nodes=...)`` with interleaved DOFs
    3 * node + component."""

    class _Dofs:
        def __init__(self, nodes, bs):
            self.nodes = np.asarray(nodes, np.int64)
            self.bs = bs
            self.nodal = {f"u^{c + 1}": bs * self.nodes + c for c in range(bs)}

        def all(self):
            return np.sort((self.bs * self.nodes[:, None] + np.arange(self.bs)).ravel())

    def __init__(self, mesh, bs=3):
        self.mesh = mesh
        self.bs = bs
        self.N = bs * mesh.p.shape[1]

    def get_dofs(self, nodes):
        return FakeBasis._Dofs(nodes, self.bs)


# --------------------------------------------------------------------------
def unit_fixtures(sk):
    from sktopt.core import derivatives, projection
    from sktopt.fea import composer
    from sktopt.mesh import utils
    from sktopt.core.optimizers import oc, logmoc
    from sktopt.filters import spacial
    from sktopt import tools
    rng = np.random.default_rng(20241204)
    out = {}
    # projection.py:27-118
    x = rng.uniform(-0.2, 1.2, 257)
    for i, (beta, eta) in enumerate([(1.0, 0.5), (2.5, 0.5), (8.0, 0.4), (32.0, 0.6)]):
        y = np.empty_like(x)
        dy = np.empty_like(x)
        projection.heaviside_projection_inplace(x, beta=beta, eta=eta, out=y)
        projection.heaviside_projection_derivative_inplace(x, beta=beta, eta=eta, out=dy)
        out[f"proj_{i}"] = y
        out[f"dproj_{i}"] = dy
        out[f"proj_param_{i}"] = np.array([beta, eta])
    out["proj_x"] = x
    # derivatives.py:25-89, composer.py:19-50
    rho = np.concatenate([rng.uniform(0.0, 1.0, 200), [0.0, 1e-7, 1e-6, 1.0]])
    en = rng.uniform(0.0, 3.0, rho.size)
    out["deriv_rho"], out["deriv_energy"] = rho, en
    for p in (1.0, 3.0, 4.5):
        k = f"{p:g}".replace(".", "_")
        out[f"E_simp_p{k}"] = derivatives._E_simp(rho, 1.0, 1e-9, p)
        out[f"E_ramp_p{k}"] = derivatives._E_ramp(rho, 1.0, 1e-9, p)
        out[f"dE_simp_p{k}"] = derivatives.dE_drho_simp(rho, 1.0, 1e-9, p)
        out[f"dE_ramp_p{k}"] = derivatives.dE_drho_ramp(rho, 1.0, 1e-9, p)
        out[f"dC_simp_p{k}"] = derivatives.dC_drho_simp(rho, en, 1.0, 1e-9, p)
        out[f"dC_ramp_p{k}"] = derivatives.dC_drho_ramp(rho, en, 1.0, 1e-9, p)
        out[f"simp_p{k}"] = composer.simp_interpolation(rho, 210e3, 210.0, p)
        out[f"ramp_p{k}"] = composer.ramp_interpolation(rho, 210e3, 210.0, p)
    E = rng.uniform(0.5, 2.0, 16)
    lam, mu = composer.lam_mu(E, 0.3)
    out["lame_E"], out["lame_lam"], out["lame_mu"] = E, lam, mu
    # composer.py:164-248: element volumes of a jittered hex grid and its tets
    mh = omesh.create_box_hex(5, 4, 3)
    ph = mh.p + rng.uniform(-0.2, 0.2, mh.p.shape)
    out["vol_hex_p"], out["vol_hex_t"] = ph, mh.t
    out["vol_hex"] = composer._get_elements_volume_hex(mh.t, ph)
    mt = omesh.create_box_tet(4, 3, 2, 1.0, 0.75, 0.5, jitter=0.15, seed=3)
    out["vol_tet_p"], out["vol_tet_t"] = mt.p, mt.t
    out["vol_tet"] = composer._get_elements_volume_tet(mt.t, mt.p)
    # mesh/utils.py:18-91: orientation fixes on shuffled connectivity
    th = mh.t.copy()
    flip = rng.random(th.shape[1]) < 0.5
    th[1, flip], th[3, flip] = mh.t[3, flip], mh.t[1, flip]
    out["orient_hex_in"] = th
    out["orient_hex_out"] = utils.fix_hexahedron_orientation(th, mh.p)
    tt = mt.t.copy()
    flip = rng.random(tt.shape[1]) < 0.5
    tt[1, flip], tt[2, flip] = mt.t[2, flip], mt.t[1, flip]
    out["orient_tet_in"] = tt
    out["orient_tet_out"] = utils.fix_tetrahedron_orientation(tt, mt.p)
    # mesh/utils.py:180-228
    fm = fake_mesh(sk, mh)
    nodes_a = np.array([0, 7, 33, 59])
    nodes_b = np.array([5, 6, 100, 119])
    out["ebn_nodes_a"], out["ebn_nodes_b"] = nodes_a, nodes_b
    out["ebn_a"] = utils.get_elements_by_nodes(fm, nodes_a)
    out["ebn_ab"] = utils.get_elements_by_nodes(fm, [nodes_a, nodes_b])
    # tools/scheduler.py: every kind through Schedulers (values_as_list)
    S = tools.SchedulerConfig
    confs = [
        ("constant", S.constant(target_value=0.3)),
        ("step", S.step(init_value=1.0, target_value=3.0, num_steps=3)),
        ("step_to_one", S.step_to_one(num_steps=4)),
        ("step_accelerating", S.step_accelerating(init_value=1.0, target_value=2.0,
                                                  num_steps=3, curvature=2.0)),
        ("step_accelerating_to_one", S.step_accelerating_to_one(num_steps=5,
                                                                curvature=3.0)),
        ("step_decelerating", S.step_decelerating(init_value=0.5, target_value=0.1,
                                                  num_steps=4, curvature=2.0)),
        ("step_decelerating_to_one", S.step_decelerating_to_one(num_steps=3,
                                                                curvature=1.5)),
        ("sawtooth_decay", S.sawtooth_decay("move_limit", 0.3, 0.1, 3)),
    ]
    iters = 37
    with tempfile.TemporaryDirectory() as d:
        sch = tools.Schedulers(d)
        for name, c in confs:
            sch.add_object_from_config(c, name)
        sch.set_iters_max(iters)
        vals = np.array([sch.values_as_list(it, [n for n, _ in confs]) for it in
                         range(0, iters + 2)], dtype=float)
    out["sched_names"] = np.array([n for n, _ in confs])
    out["sched_iters_max"] = np.array(iters)
    out["sched_values"] = vals
    # filters/spacial.py:19-166 on a 10x5x4 grid with a design mask
    mg = omesh.create_box_hex(10, 5, 4)
    design_mask = np.ones(mg.nelements, bool)
    design_mask[rng.choice(mg.nelements, 23, replace=False)] = False
    fmg = fake_mesh(sk, mg)
    vol = np.ones(mg.nelements)
    xv = rng.uniform(0.0, 1.0, mg.nelements)
    out["filt_x"], out["filt_design_mask"] = xv, design_mask
    for i, r in enumerate((1.5, 2.2)):
        f = spacial.SpacialFilter.from_defaults(fmg, vol, r, design_mask=design_mask)
        y = f.forward(xv)
        g = f.gradient(xv)
        W = f.W.tocsr()
        W.sort_indices()
        out[f"filt_r{i}"] = np.array(r)
        out[f"filt_fwd_{i}"], out[f"filt_grad_{i}"] = y, g
        out[f"filt_W_indptr_{i}"], out[f"filt_W_indices_{i}"] = W.indptr, W.indices
        out[f"filt_W_data_{i}"] = W.data
    # oc.py:16-95 bisection, with the reference filter at r = 1.5
    f = spacial.SpacialFilter.from_defaults(fmg, vol, 1.5, design_mask=design_mask)
    design = np.nonzero(design_mask)[0]
    nd = design.size
    rho_full = np.ones(mg.nelements)
    rho_full[design] = rng.uniform(0.05, 0.9, nd)
    rho_e = rho_full[design].copy()
    dC = -rng.uniform(0.01, 1.0, nd)
    ev = rng.uniform(0.8, 1.2, nd)
    bufs = [np.empty(nd) for _ in range(4)] + [np.empty(mg.nelements) for _ in range(3)]
    lmid, verr = oc.bisection_with_physical_volume(
        dC, rho_e, rho_full, design, f, 1e-2, 1.0, 0.2, 0.5, 1e-12, 0.35, 2.0, 0.5,
        bufs[0], bufs[1], bufs[2], bufs[3], ev, float(np.sum(ev)), 0.7, 1.3,
        bufs[4], bufs[5], bufs[6], max_iter=1000, tolerance=1e-5, l1=1e-7, l2=1e7)
    out.update(bis_design=design, bis_rho_full=rho_full, bis_dC=dC, bis_vol=ev,
               bis_lmid=np.array(lmid), bis_vol_error=np.array(verr),
               bis_scaling_rate=bufs[0].copy(), bis_rho_design=bufs[1].copy(),
               bis_clip_lower=bufs[2].copy(), bis_clip_upper=bufs[3].copy(),
               bis_params=np.array([1e-2, 1.0, 0.2, 0.5, 1e-12, 0.35, 2.0, 0.5, 0.7, 1.3,
                                    1e-5, 1e-7, 1e7]))
    # logmoc.py:36-66
    rl = np.concatenate([rng.uniform(0.0, 1.0, 300), [0.0, 1.0, 2.0]])
    dL = rng.normal(0.0, 1.5, rl.size)
    r_io = rl.copy()
    sr, lo, up = np.empty_like(rl), np.empty_like(rl), np.empty_like(rl)
    logmoc.lagrangian_log_update(r_io, dL, sr, 0.5, 0.2, lo, up, 1e-2, 1.0, 1.0)
    out.update(llu_rho_in=rl, llu_dL=dL, llu_rho_out=r_io, llu_scaling_rate=sr,
               llu_lower=lo, llu_upper=up, llu_params=np.array([0.5, 0.2, 1e-2, 1.0, 1.0]))
    return out


# --------------------------------------------------------------------------
class CachedSpacialFilter:
    """Wraps the reference SpacialFilter and reuses its matrix while the
    radius is unchanged (the reference rebuilds an identical matrix on every
    forward call)."""

    def __init__(self, inner):
        self.inner = inner
        self._r = None

    def __getattr__(self, k):
        return getattr(self.inner, k)

    @property
    def radius(self):
        return self.inner.radius

    def update_radius(self, r, **a):
        self.inner.update_radius(r, **a)

    def forward(self, rho):
        if self._r != self.inner.radius:
            y = self.inner.forward(rho)
            self._r = self.inner.radius
            return y
        out = np.copy(rho)
        m = self.inner.design_mask
        out[m] = self.inner.W @ rho[m]
        return out

    def gradient(self, v):
        return self.inner.gradient(v)


class OracleFEM:
    """FEM plugin with the reference interface (solver_elastic.py:619-676)
    over the oracle's restated scikit-fem arithmetic."""

    def __init__(self, pb, E0, Emin_coeff, solver="spsolve", rtol=1e-8):
        self.pb, self.E0, self.Emin = pb, E0, E0 * Emin_coeff
        self.solver, self.rtol = solver, rtol
        self.solve_s = 0.0

    def objectives_multi_load(self, rho, p, u_dofs, timer=None, force_scale=1.0):
        t0 = time.perf_counter()
        comp, U = self.pb.objectives(rho, p, self.Emin, self.solver, self.rtol,
                                     force_scale=force_scale)
        self.solve_s += time.perf_counter() - t0
        u_dofs[:] = U
        return comp

    def energy_multi_load(self, rho, p, u_dofs):
        return self.pb.energy(rho, p, self.Emin, u_dofs)


def reference_task(sk, m, dir_nodes, load_nodes, forces, E0, nu):
    """sktopt.mesh.LinearElasticity through the reference's FEMDomain.from_nodes
    (design sets, fixed and Dirichlet/Neumann elements, element volumes)."""
    from sktopt.mesh.task_common import FEMDomain
    from sktopt.mesh.task_elastic import LinearElasticity
    basis = FakeBasis(fake_mesh(sk, m))
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        base = FEMDomain.from_nodes(basis, dir_nodes, "all", None, load_nodes, "u^3", -1.0,
                                    None, None, None, None, None,
                                    np.arange(m.nelements))
    fields = [getattr(base, k) for k in (
        "basis", "dirichlet_nodes", "dirichlet_dofs", "dirichlet_elements",
        "dirichlet_values", "neumann_nodes", "neumann_elements", "neumann_dir_type",
        "neumann_values", "robin_facets_ids", "robin_nodes", "robin_elements",
        "robin_coefficient", "robin_bc_value", "design_robin_boundary", "design_elements",
        "free_dofs", "free_elements", "all_elements", "fixed_elements",
        "dirichlet_neumann_elements", "elements_volume")]
    return LinearElasticity(*fields, E0, nu, [np.asarray(f, float) for f in forces])


def _silence(opt):
    """No files besides the density npz: VTU, images and plots are skipped."""
    from sktopt.core import visualization
    from sktopt.mesh import visualization as vmesh
    visualization.export_mesh_with_info = lambda *a, **k: None
    visualization.rho_histo_plot = lambda *a, **k: None
    vmesh.export_submesh = lambda *a, **k: None
    opt.tsk.export_analysis_condition_on_mesh = lambda *a, **k: None
    opt._save_timing_plot = lambda *a, **k: None
    opt._report_timing = lambda *a, **k: None
    opt.recorder.print = lambda *a, **k: None
    opt.recorder.export_progress = lambda *a, **k: None
    opt.recorder.export_histories = lambda *a, **k: None
    opt.schedulers.export = lambda *a, **k: None


def run_reference_loop(sk, method, size, iters, cfg_kw, snap_iters=(), load_frac=None,
                       solver="spsolve"):
    """The reference driver (common_density.py:966-1243) on the cantilever of
    `size` for `iters` iterations.  Returns per-iteration histories and the
    density after each iteration in `snap_iters`."""
    import sktopt
    m, pb, design_o, fixed_o, vol_o = problems.cantilever(*size, load_frac=load_frac)
    dir_nodes, load_nodes = problems.cantilever_sets(m, load_frac)
    tsk = reference_task(sk, m, dir_nodes, load_nodes, pb.forces, 1.0, 0.3)
    with tempfile.TemporaryDirectory() as d:
        if method == "oc":
            cfg = sktopt.core.optimizers.OC_Config(**cfg_kw)
            cls = sktopt.core.OC_Optimizer
        else:
            cfg = sktopt.core.optimizers.LogMOC_Config(**cfg_kw)
            cls = sktopt.core.LogMOC_Optimizer
        cfg.max_iters = iters
        cfg.record_times = iters
        cfg.dst_path = d
        opt = cls(cfg, tsk)
        fem = OracleFEM(pb, 1.0, cfg.E_min_coeff, solver=solver)
        opt.fem = fem
        opt.parameterize()
        opt.filter = CachedSpacialFilter(opt.filter)
        _silence(opt)
        snaps = {}
        t0 = time.perf_counter()
        for it in range(1, iters + 1):
            opt.optimize_steps(1)
            if it in snap_iters:
                snaps[f"rho_it{it}"] = opt._state.rho.copy()
        wall = time.perf_counter() - t0
        H = opt.recorder.as_object()
        out = {"size": np.array(size), "iters": np.array(iters),
               "design": np.asarray(tsk.design_elements),
               "dirichlet_neumann_elements": np.asarray(tsk.dirichlet_neumann_elements),
               "compliance": np.array(H.compliance, float),
               "vol_error": np.array(H.vol_error, float),
               "kkt_residual": np.array(H.kkt_residual, float),
               "rho_final": opt._state.rho.copy(),
               "rho_projected_final": opt._state.rho_projected.copy(),
               "wall_s": np.array(wall), "solve_s": np.array(fem.solve_s)}
        if hasattr(H, "lmid"):
            out["lmid"] = np.array(H.lmid, float)
        if hasattr(H, "lambda_v"):
            out["lambda_v"] = np.array(H.lambda_v, float)
        out.update(snaps)
    return out


def rho_update_fixtures(sk):
    """OC_Optimizer.rho_update (oc.py:149-250) and LogMOC_Optimizer.rho_update
    (logmoc.py:90-258) called exactly as the driver calls them
    (common_density.py:1112-1129), twice in a row, on seeded inputs over the
    12x6x6 cantilever with the reference SpacialFilter (r = 1.5)."""
    import sktopt
    from sktopt.core.optimizers.common_density import DensityState  # noqa: F401
    m, pb, design_o, fixed_o, vol_o = problems.cantilever(12, 6, 6)
    dir_nodes, load_nodes = problems.cantilever_sets(m)
    ne = m.nelements
    rng = np.random.default_rng(99)
    out = {}
    for method in ("oc", "logmoc"):
        tsk = reference_task(sk, m, dir_nodes, load_nodes, pb.forces, 1.0, 0.3)
        with tempfile.TemporaryDirectory() as d:
            if method == "oc":
                cfg = sktopt.core.optimizers.OC_Config(
                    filter_type="spacial", percentile=sktopt.tools.SchedulerConfig.none())
                cls = sktopt.core.OC_Optimizer
            else:
                cfg = sktopt.core.optimizers.LogMOC_Config(filter_type="spacial")
                cls = sktopt.core.LogMOC_Optimizer
            cfg.dst_path = d
            cfg.filter_radius = sktopt.tools.SchedulerConfig.constant(target_value=1.5)
            opt = cls(cfg, tsk)
            opt.parameterize()
            opt.filter.update_radius(1.5)
            _silence(opt)
            # DensityMethod.__init__ removed the Dirichlet elements from the
            # design set (design_dirichlet False, task_common.py:398-401)
            design = np.asarray(tsk.design_elements)
            nd = design.size
            out["design"] = design
            out["dirichlet_neumann_elements"] = np.asarray(tsk.dirichlet_neumann_elements)
            rho = np.ones(ne)
            rho[design] = rng.uniform(0.05, 0.95, nd)
            opt._state = types.SimpleNamespace(rho=rho, rho_filtered=None)
            ev = tsk.elements_volume[design]
            evs = float(np.sum(ev))
            for call, (it, move, eta, beta, vf, pct) in enumerate(
                    [(1, 0.2, 0.5, 1.0, 0.3, None), (2, 0.15, 0.5, 1.5, 0.3, 90.0)]):
                rho_f = opt.filter.forward(rho)
                rho_p = np.empty(ne)
                sktopt.core.projection.heaviside_projection_inplace(
                    rho_f, beta=beta, eta=cfg.beta_eta, out=rho_p)
                opt._state.rho_filtered = rho_f
                dC = -rng.uniform(0.01, 2.0, nd) * (1.0 + 3.0 * rho[design] ** 2)
                rde = rho[design].copy()
                sr = np.zeros(nd)
                lo, up = np.zeros(nd), np.zeros(nd)
                pre = dict(rho=rho.copy(), rho_filtered=rho_f.copy(), rho_projected=rho_p,
                           dC=dC.copy(), rho_design=rde.copy())
                opt.rho_update(it, rde, rho_p, dC, None, None, sr, move, eta, beta, lo, up,
                               pct, ev, evs, vf)
                k = f"{method}_{call}"
                for name, v in pre.items():
                    out[f"{k}_in_{name}"] = v
                out[f"{k}_params"] = np.array([it, move, eta, beta, vf,
                                               -1.0 if pct is None else pct])
                out[f"{k}_out_rho_design"] = rde.copy()
                out[f"{k}_out_dC"] = dC.copy()
                out[f"{k}_out_scaling_rate"] = sr.copy()
                out[f"{k}_out_clip_lower"] = lo.copy()
                out[f"{k}_out_clip_upper"] = up.copy()
                out[f"{k}_out_running_scale"] = np.array(opt.running_scale)
                out[f"{k}_out_kkt"] = np.array(opt.kkt_residual)
                out[f"{k}_out_vol_error"] = np.array(opt.recorder.latest("vol_error"))
                if method == "oc":
                    out[f"{k}_out_lmid"] = np.array(opt.recorder.latest("lmid"))
                else:
                    out[f"{k}_out_lambda_v"] = np.array(opt.lambda_v)
                rho[design] = rde
                rho[tsk.dirichlet_neumann_elements] = 1.0
    return out


def config_defaults(sk):
    """Field defaults of OC_Config, LogMOC_Config (with DensityMethodConfig's
    through inheritance) and LinearSolverConfig; schedules as their fields."""
    import dataclasses
    import sktopt
    from sktopt.fea.solver_elastic import LinearSolverConfig

    def enc(v):
        if dataclasses.is_dataclass(v):
            return {f.name: enc(getattr(v, f.name)) for f in dataclasses.fields(v)}
        if isinstance(v, (bool, int, float, str)) or v is None:
            return v
        return repr(v)
    out = {}
    for name, cls in (("OC_Config", sktopt.core.optimizers.OC_Config),
                      ("LogMOC_Config", sktopt.core.optimizers.LogMOC_Config),
                      ("LinearSolverConfig", LinearSolverConfig)):
        c = cls()
        out[name] = {f.name: enc(getattr(c, f.name)) for f in dataclasses.fields(c)
                     if f.name not in ("petsc_options",)}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--c1", action="store_true")
    args = ap.parse_args()
    sk = import_reference()
    import sktopt
    SC = sktopt.tools.SchedulerConfig
    import json
    with open(os.path.join(HERE, "ref_config_defaults.json"), "w") as f:
        json.dump(config_defaults(sk), f, indent=1, sort_keys=True)
    t = time.perf_counter()
    np.savez_compressed(os.path.join(HERE, "ref_units.npz"), **unit_fixtures(sk))
    print(f"ref_units.npz ({time.perf_counter() - t:.1f} s)")
    t = time.perf_counter()
    np.savez_compressed(os.path.join(HERE, "ref_rho_update.npz"), **rho_update_fixtures(sk))
    print(f"ref_rho_update.npz ({time.perf_counter() - t:.1f} s)")
    # the benchmark cantilever settings (60x20x20 / 240x80x80 workloads)
    bench_kw = dict(filter_type="spacial", filter_radius=SC.constant(target_value=1.5),
                    p=SC.constant(target_value=3.0), vol_frac=SC.constant(target_value=0.3),
                    move_limit=SC.constant(target_value=0.2), E_min_coeff=1e-9)
    t = time.perf_counter()
    np.savez_compressed(os.path.join(HERE, "ref_loop_oc_12x6x6.npz"),
                        **run_reference_loop(sk, "oc", (12, 6, 6), 6, bench_kw,
                                             snap_iters=(1, 3)))
    print(f"ref_loop_oc_12x6x6.npz ({time.perf_counter() - t:.1f} s)")
    # reference defaults (p and beta continuation, sawtooth move limit, vf
    # 0.8, Emin 1e-3) with the spacial filter, a load at y = 0.25 ny
    t = time.perf_counter()
    np.savez_compressed(os.path.join(HERE, "ref_loop_oc_defaults_10x5x4.npz"),
                        **run_reference_loop(sk, "oc", (10, 5, 4), 8,
                                             dict(filter_type="spacial",
                                                  filter_radius=SC.constant(target_value=1.2)),
                                             load_frac=0.25))
    print(f"ref_loop_oc_defaults_10x5x4.npz ({time.perf_counter() - t:.1f} s)")
    # the optional sensitivity filter (common_density.py:1102-1106)
    t = time.perf_counter()
    np.savez_compressed(os.path.join(HERE, "ref_loop_oc_sensfilter_12x6x6.npz"),
                        **run_reference_loop(sk, "oc", (12, 6, 6), 5,
                                             dict(bench_kw, sensitivity_filter=True)))
    print(f"ref_loop_oc_sensfilter_12x6x6.npz ({time.perf_counter() - t:.1f} s)")
    t = time.perf_counter()
    np.savez_compressed(os.path.join(HERE, "ref_loop_logmoc_12x6x6.npz"),
                        **run_reference_loop(sk, "logmoc", (12, 6, 6), 6,
                                             dict(bench_kw, vol_frac=SC.constant(
                                                 target_value=0.4)),
                                             snap_iters=(1, 3)))
    print(f"ref_loop_logmoc_12x6x6.npz ({time.perf_counter() - t:.1f} s)")
    if args.c1:
        t = time.perf_counter()
        # direct solves with the minimum-degree ordering (oracle solver
        # "spsolve_mmd"): the reference's default COLAMD ordering takes
        # minutes per solve at this size
        res = run_reference_loop(sk, "oc", (60, 20, 20), 30, bench_kw, snap_iters=(10,),
                                 solver="spsolve_mmd")
        keep = {k: v for k, v in res.items() if k not in ("rho_final", "rho_projected_final",
                                                         "design",
                                                         "dirichlet_neumann_elements")}
        np.savez_compressed(os.path.join(HERE, "ref_loop_oc_60x20x20.npz"), **keep)
        print(f"ref_loop_oc_60x20x20.npz ({time.perf_counter() - t:.1f} s)")


if __name__ == "__main__":
    main()
