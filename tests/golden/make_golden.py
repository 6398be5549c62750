"""Generate the golden fixtures from the CPU oracle (oracle/).

The reference (scikit-topt 0.3.9) cannot be imported here (scikit-fem, PyAMG
and numba are missing), so the fixtures pin the oracle -- the NumPy/SciPy
restatement of the reference algorithm -- against future drift, and give the
GPU tests a stored target.  Run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import fem as ofem          # noqa: E402
from oracle import filters as ofilt     # noqa: E402
from oracle import optim as oopt        # noqa: E402
from oracle import problems             # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def cantilever_state(nx=10, ny=5, nz=4, seed=7):
    m, pb, design, fixed, vol = problems.cantilever(nx, ny, nz)
    rho = np.random.default_rng(seed).uniform(0.01, 1.0, m.nelements)
    K = pb.stiffness(rho, 3.0, 1e-9)
    F = np.column_stack(pb.forces)
    Ke, Fe = ofem.enforce(K, F, pb.dirichlet_dofs)
    U = ofem.solve(Ke, Fe[:, 0], "spsolve")[:, None]
    comp = float(Fe[:, 0] @ U[:, 0])
    energy = pb.energy(rho, 3.0, 1e-9, U)[:, 0]
    dc = ofem.dC_drho_simp(rho, energy, 1.0, 1e-9, 3.0)
    mask = np.zeros(m.nelements, bool)
    mask[design] = True
    filt = ofilt.SpacialFilter(m, 1.5, mask)
    x = np.random.default_rng(seed + 1).uniform(0.0, 1.0, m.nelements)
    return dict(
        shape=np.array([nx, ny, nz]), rho=rho, K_indptr=Ke.indptr, K_indices=Ke.indices,
        K_data=Ke.data, F=Fe, U=U, compliance=comp, energy=energy, dc=dc,
        design=np.asarray(design), W_indptr=filt.W.indptr, W_indices=filt.W.indices,
        W_data=filt.W.data, filt_x=x, filt_fwd=filt.forward(x), filt_grad=filt.gradient(x),
        proj_b125=ofilt.heaviside_projection(x, 1.25, 0.5),
        dproj_b125=ofilt.heaviside_projection_derivative(x, 1.25, 0.5))


def oc_trajectory(nx=12, ny=6, nz=6, n_iter=5):
    m, pb, design, fixed, vol = problems.cantilever(nx, ny, nz)
    filt = problems.gaussian_filter_for(m, design, 1.5)
    cfg = oopt.OracleConfig(max_iters=n_iter, p=oopt.Sched("Constant", 3.0, 3.0),
                            vol_frac=oopt.Sched("Constant", 0.3, 0.3),
                            move_limit=oopt.Sched("Constant", 0.2, 0.2),
                            filter_radius=oopt.Sched("Constant", 1.5, 1.5), E_min_coeff=1e-9)
    opt = oopt.OracleOptimizer(cfg, pb, filt, design, fixed, vol)
    rhos = []
    for _ in range(n_iter):
        opt.step()
        rhos.append(opt.rho.copy())
    h = opt.hist
    return dict(shape=np.array([nx, ny, nz]), compliance=np.array(h["compliance"]),
                lmid=np.array(h["lmid"]), vol_error=np.array(h["vol_error"]),
                kkt=np.array(h["kkt_residual"]), steps=np.array(h["bisection_steps"]),
                rho=np.array(rhos))


def heat_plate_state(nx=12, ny=12, nz=3, seed=11):
    """The heat task of the reference's flow test on an nx x ny x nz plate:
    objectives, temperatures, adjoints, energies and sensitivities for the
    three objectives (heat exchange with avg_temp_weight 0.5)."""
    from oracle import heat_robin as hr
    out = {"shape": np.array([nx, ny, nz])}
    rho = None
    for obj, w in (("compliance", 0.0), ("heat_exchange", 0.5), ("averaged_temp", 0.0)):
        m, pb, *_ = problems.heat_plate(nx, ny, nz, objective=obj, avg_temp_weight=w)
        if rho is None:
            rho = np.random.default_rng(seed).uniform(0.1, 1.0, m.nelements)
            out["rho"] = rho
            out["rho_nodal"] = hr.nodal_average(m, rho, "reference")[0]
        J, T = pb.objectives(rho, 3.0, 1e-2)
        out[f"{obj}_J"] = J
        out[f"{obj}_T"] = T
        if pb.lam is not None:
            out[f"{obj}_lam"] = pb.lam
        out[f"{obj}_energy"] = pb.energy(rho, 3.0, 1e-2, T)
        out[f"{obj}_dc"] = pb.custom_sensitivity(rho, 3.0, 1e-2, T)
    return out


def tet_tractions(seed=4):
    """Boundary facets and two traction load cases on a jittered tet box."""
    from oracle import surface as osurf
    from oracle import mesh as omesh
    m = omesh.create_box_tet(5, 3, 3, 2.0, 1.0, 1.0, jitter=0.25, seed=seed)
    f1 = osurf.boundary_facets(m, problems.in_range((2.0, 2.0), (0, 9), (0, 9)))
    f2 = osurf.boundary_facets(m, problems.in_range((0, 2.0), (1.0, 1.0), (0, 9)))
    F = osurf.surface_forces(m, [f1, f2], ["u^3", "u^1"], [-2.0, 0.5])
    return dict(p=m.p, t=m.t, facets1=f1, facets2=f2, F1=F[0], F2=F[1])


FIXTURES = {
    "cantilever_10x5x4_state.npz": cantilever_state,
    "cantilever_12x6x6_oc5.npz": oc_trajectory,
    "heat_plate_12x12x3.npz": heat_plate_state,
    "tet_tractions.npz": tet_tractions,
}


def main(names=None):
    """Write the fixtures named on the command line (default: all)."""
    for name in (names or FIXTURES):
        np.savez_compressed(os.path.join(HERE, name), **FIXTURES[name]())
        print("wrote", name)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
