"""GPU parity of assembly, enforcement, SpMV, PCG solves and energies against
the CPU oracle (SciPy CSR + spsolve).

Tolerances: assembled values 1e-13 relative to max |K|; FP64 PCG compliance
1e-10 relative (solver rtol 1e-12); mixed refined compliance 1e-6 relative
(displacements 1e-6 of max |U|); matrix-free FP32 operator 2e-6 of max |y|;
energies and sensitivities 1e-9 relative L2 (they inherit the solve error).
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import fem as ofem
from oracle import mesh as omesh
from oracle import problems

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda", 0)


def _engine_for(tsk, mixed=False, multigrid=True):
    from sktopt_gb300.fea import composer
    from sktopt_gb300.fea.engine import FemEngine
    Ke, Kh, _ = composer.element_matrices(tsk.mesh, getattr(tsk, "nu", 0.3))
    ke = Ke if tsk.bs == 3 else Kh
    return FemEngine(tsk.mesh, tsk.bs, ke, tsk.dirichlet_mask, mixed=mixed,
                     multigrid=multigrid)


def _rho(n, seed=0, lo=0.05):
    return np.random.default_rng(seed).uniform(lo, 1.0, n)


@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_assembly_matches_oracle_csr(native_lib, kind):
    import torch
    from sktopt_gb300.fea.engine import block_to_scalar_csr, pattern
    from sktopt_gb300.mesh import toy_problem
    if kind == "hex":
        tsk = toy_problem.cantilever(6, 4, 3)
        om = omesh.create_box_hex(6, 4, 3)
    else:
        tsk = toy_problem.multi_load_tet(4, 3, 2, 2.0, 1.0, 1.0, jitter=0.2, seed=5)
        om = omesh.create_box_tet(4, 3, 2, 2.0, 1.0, 1.0, jitter=0.2, seed=5)
    rho = _rho(tsk.mesh.nelements)
    eng = _engine_for(tsk, multigrid=False)
    eng.update(torch.from_numpy(rho).to(_dev()), 1.0, 1e-9, 3.0)
    vals = eng.export_values().cpu().numpy()
    rp, ci, _, _ = pattern(tsk.mesh)
    ip, idx, dat = block_to_scalar_csr(rp, ci, vals, 3)
    if kind == "hex":
        Kl = ofem.hex_element_matrices(om.p[:, om.t[:, 0]], 0.3)[0]
    else:
        Kl = ofem.element_matrices(om, 0.3)[0]
    K = ofem.assemble(om.t, Kl, ofem.simp_interpolation(rho, 1.0, 1e-9, 3.0), om.nnodes, 3)
    Ke_, _ = ofem.enforce(K, np.zeros(K.shape[0]), tsk.dirichlet_dofs)
    assert np.array_equal(ip, Ke_.indptr) and np.array_equal(idx, Ke_.indices)
    np.testing.assert_allclose(dat, Ke_.data, rtol=0, atol=1e-13 * np.abs(Ke_.data).max())


def test_spmv_f64_and_f32(native_lib):
    import torch
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(8, 4, 4)
    rho = _rho(tsk.mesh.nelements, 1)
    m, pb, *_ = problems.cantilever(8, 4, 4)
    K = pb.stiffness(rho, 3.0, 1e-9)
    Ke_, _ = ofem.enforce(K, np.zeros(K.shape[0]), pb.dirichlet_dofs)
    x = np.random.default_rng(2).standard_normal((K.shape[0], 3))
    for mixed in (False, True):
        eng = _engine_for(tsk, mixed=mixed)
        eng.update(torch.from_numpy(rho).to(_dev()), 1.0, 1e-9, 3.0)
        y = eng.spmv(torch.from_numpy(x).to(_dev())).cpu().numpy()
        ref = Ke_ @ x
        np.testing.assert_allclose(y, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
        if mixed:
            y32 = eng.spmv(torch.from_numpy(x).float().to(_dev()), torch.float32).cpu().numpy()
            np.testing.assert_allclose(y32, ref, rtol=0, atol=2e-5 * np.abs(ref).max())


@pytest.mark.parametrize("precond", [0, 1])
def test_fp64_pcg_compliance_vs_spsolve(native_lib, precond):
    import torch
    from sktopt_gb300.mesh import toy_problem
    nx, ny, nz = 12, 6, 6
    tsk = toy_problem.cantilever(nx, ny, nz)
    m, pb, *_ = problems.cantilever(nx, ny, nz)
    rho = _rho(tsk.mesh.nelements, 3, lo=1e-3)
    comp_ref, U_ref = pb.objectives(rho, 3.0, 1e-9, "spsolve")
    eng = _engine_for(tsk, multigrid=(precond == 1))
    dev = _dev()
    eng.update(torch.from_numpy(rho).to(dev), 1.0, 1e-9, 3.0)
    F = torch.from_numpy(np.column_stack(tsk.neumann_linear)).to(dev)
    U = torch.zeros_like(F)
    comp, st = eng.solve(F, U, 0, precond, 1e-12, 20000)
    assert st.status == 0, st
    assert abs(comp[0] - comp_ref[0]) <= 1e-10 * abs(comp_ref[0])
    np.testing.assert_allclose(U.cpu().numpy(), U_ref, rtol=0,
                               atol=1e-8 * np.abs(U_ref).max())


def test_mixed_refined_compliance(native_lib):
    import torch
    from sktopt_gb300.mesh import toy_problem
    nx, ny, nz = 16, 8, 8
    tsk = toy_problem.cantilever(nx, ny, nz)
    m, pb, *_ = problems.cantilever(nx, ny, nz)
    rho = _rho(tsk.mesh.nelements, 4, lo=1e-3)
    comp_ref, U_ref = pb.objectives(rho, 3.0, 1e-9, "spsolve")
    dev = _dev()
    eng = _engine_for(tsk, mixed=True)
    eng.update(torch.from_numpy(rho).to(dev), 1.0, 1e-9, 3.0)
    F = torch.from_numpy(np.column_stack(tsk.neumann_linear)).to(dev)
    U = torch.zeros_like(F)
    # 1 reliable updates, 2 restarted refinement, 3 flexible CG with the FP64
    # operator, 4 flexible CG with the FP32 operator and residual replacement
    for method in (1, 2, 3, 4):
        comp, st = eng.solve(F, U, method, 1, 1e-8, 500,
                             inner_rtol=1e-4 if method == 2 else 1e-1)
        assert st.status == 0, (method, st)
        assert st.outer >= 1
        assert st.relres <= 1e-8
        assert abs(comp[0] - comp_ref[0]) <= 1e-6 * abs(comp_ref[0]), method
        np.testing.assert_allclose(U.cpu().numpy(), U_ref, rtol=0,
                                   atol=1e-6 * np.abs(U_ref).max())


@pytest.mark.parametrize("ny", [10, 26, 31])   # node tiles 16, 27 and 32 nodes high
def test_matrix_free_operator_matches_assembled(native_lib, ny):
    """FP32 matrix-free operator of a uniform hex grid vs the assembled FP32
    matrix (same enforced operator, FP32 rounding apart)."""
    import torch
    from sktopt_gb300.fea import composer
    from sktopt_gb300.fea.engine import FemEngine
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(9, ny, 5)
    Ke, _, _ = composer.element_matrices(tsk.mesh, 0.3)
    rho = torch.from_numpy(_rho(tsk.mesh.nelements, 11, lo=1e-3)).to(_dev())
    x = torch.from_numpy(np.random.default_rng(12).standard_normal((3 * tsk.mesh.nnodes, 1)))
    x32 = x.float().to(_dev())
    out = []
    for mf in (True, False):
        eng = FemEngine(tsk.mesh, 3, Ke, tsk.dirichlet_mask, mixed=True, multigrid=True,
                        matrix_free=mf)
        eng.update(rho, 1.0, 1e-9, 3.0)
        out.append(eng.spmv(x32, torch.float32).double().cpu().numpy())
    ref = out[1]
    np.testing.assert_allclose(out[0], ref, rtol=0, atol=2e-6 * np.abs(ref).max())


def test_energy_and_sensitivity(native_lib):
    import torch
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(10, 5, 4)
    m, pb, *_ = problems.cantilever(10, 5, 4)
    rho = _rho(tsk.mesh.nelements, 6, lo=0.01)
    comp_ref, U_ref = pb.objectives(rho, 3.0, 1e-9, "spsolve")
    en_ref = pb.energy(rho, 3.0, 1e-9, U_ref)
    dc_ref = ofem.dC_drho_simp(rho, en_ref[:, 0], 1.0, 1e-9, 3.0)
    dev = _dev()
    eng = _engine_for(tsk)
    rt = torch.from_numpy(rho).to(dev)
    eng.update(rt, 1.0, 1e-9, 3.0)
    U = torch.from_numpy(np.ascontiguousarray(U_ref)).to(dev)
    en, dc = eng.energy(U, rt, 1.0, 1e-9, 3.0, want_dc=True)
    # u_e^T K0 u_e cancels the rigid-body part of u_e, so both sides carry
    # rounding of order eps * |u_e|^2 |K0|: compare with a relative L2 bound.
    en_g = en.cpu().numpy()
    assert np.linalg.norm(en_g - en_ref) <= 1e-9 * np.linalg.norm(en_ref)
    dc_g = dc.cpu().numpy()[:, 0]
    assert np.linalg.norm(dc_g - dc_ref) <= 1e-9 * np.linalg.norm(dc_ref)


def test_multi_load_block_rhs(native_lib):
    import torch
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.multi_load_tet(6, 4, 3, 2.0, 1.0, 1.0, jitter=0.2, seed=2)
    om = omesh.create_box_tet(6, 4, 3, 2.0, 1.0, 1.0, jitter=0.2, seed=2)
    Kl = ofem.element_matrices(om, 0.3)[0]
    rho = _rho(tsk.mesh.nelements, 8, lo=0.05)
    K = ofem.assemble(om.t, Kl, ofem.simp_interpolation(rho, 1.0, 1e-9, 3.0), om.nnodes, 3)
    F = np.column_stack(tsk.neumann_linear)
    Ke_, Fe = ofem.enforce(K, F, tsk.dirichlet_dofs)
    U_ref = ofem.solve(Ke_, Fe, "spsolve")
    comp_ref = np.einsum("ij,ij->j", Fe, U_ref)
    dev = _dev()
    for mixed, method, tol in ((False, 0, 1e-10), (True, 1, 1e-6), (True, 3, 1e-6),
                               (True, 4, 1e-6)):
        eng = _engine_for(tsk, mixed=mixed)
        eng.update(torch.from_numpy(rho).to(dev), 1.0, 1e-9, 3.0)
        Ft = torch.from_numpy(np.ascontiguousarray(F)).to(dev)
        U = torch.zeros_like(Ft)
        comp, st = eng.solve(Ft, U, method, 1, 1e-12 if method == 0 else 1e-9, 5000)
        assert st.status == 0, st
        np.testing.assert_allclose(comp, comp_ref, rtol=tol)
