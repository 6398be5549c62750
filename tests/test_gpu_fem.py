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
    """FP32 matrix-free operator of a uniform hex grid -- the tensor-core
    kernel (3xTF32) and the FP32-FMA kernel -- vs the assembled FP32 matrix
    (same enforced operator, FP32 rounding apart)."""
    _mf_vs_assembled((9, ny, 5), seed=11)


@pytest.mark.parametrize("shape", [(3, 1, 1), (2, 3, 1), (30, 14, 12), (61, 20, 9),
                                   (7, 16, 33)])
def test_matrix_free_tensor_core_operator_shapes(native_lib, shape):
    """Ragged node columns (15 x 7 nodes per column) and z segments, a grid
    one cell thick, and grids one column wide or tall."""
    _mf_vs_assembled(shape, seed=sum(shape))


def _mf_vs_assembled(shape, seed):
    import torch
    from sktopt_gb300.fea import composer
    from sktopt_gb300.fea.engine import FemEngine
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(*shape)
    Ke, _, _ = composer.element_matrices(tsk.mesh, 0.3)
    rho = torch.from_numpy(_rho(tsk.mesh.nelements, seed, lo=1e-3)).to(_dev())
    x = torch.from_numpy(np.random.default_rng(seed + 1).standard_normal(
        (3 * tsk.mesh.nnodes, 1)))
    x32 = x.float().to(_dev())
    sell = FemEngine(tsk.mesh, 3, Ke, tsk.dirichlet_mask, mixed=True, multigrid=True,
                     matrix_free=False)
    sell.update(rho, 1.0, 1e-9, 3.0)
    ref = sell.spmv(x32, torch.float32).double().cpu().numpy()
    eng = FemEngine(tsk.mesh, 3, Ke, tsk.dirichlet_mask, mixed=True, multigrid=True,
                    matrix_free=True)
    eng.update(rho, 1.0, 1e-9, 3.0)
    outs = {}
    for kind in (1, 0):
        eng.set_mf_kernel(kind)
        outs[kind] = eng.spmv(x32, torch.float32).double().cpu().numpy()
        np.testing.assert_allclose(outs[kind], ref, rtol=0, atol=2e-6 * np.abs(ref).max())
    assert eng.mf_error() == 0
    # deterministic: a second product gives the same bits
    eng.set_mf_kernel(1)
    again = eng.spmv(x32, torch.float32).double().cpu().numpy()
    assert np.array_equal(again, outs[1])


def test_mixed_solve_tensor_core_operator_matches_fma(native_lib):
    """The mixed solve (every operator mode: products, residuals b - Ax and
    y - Ax inside the V-cycle, products with the p.q dot) with the tensor-core
    operator against the FP32-FMA operator: same converged compliance, same
    number of flexible-CG iterations to within two."""
    import torch
    from sktopt_gb300.fea.solver_elastic import FEM_SimpLinearElasticity, LinearSolverConfig
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(40, 16, 14)
    rho = torch.from_numpy(_rho(tsk.mesh.nelements, 21, lo=1e-3)).to(_dev())
    res = {}
    for kind in (1, 0):
        fem = FEM_SimpLinearElasticity(tsk, 1e-9, solver_config=LinearSolverConfig(
            solver="cg_pyamg", rtol=1e-8, precision="mixed"), device=_dev())
        fem.build(rho, 3.0)
        fem.engine.set_mf_kernel(kind)
        U = torch.zeros((tsk.n_dof, 1), dtype=torch.float64, device=_dev())
        comp = fem.solve_built(U)
        st = fem.solve_history[-1]
        res[kind] = (float(comp[0]), st.iters, U.cpu().numpy())
        assert fem.engine.mf_error() == 0
    (c1, it1, u1), (c0, it0, u0) = res[1], res[0]
    assert abs(c1 - c0) <= 1e-9 * abs(c0)
    assert abs(it1 - it0) <= 2, (it1, it0)
    assert np.linalg.norm(u1 - u0) <= 1e-7 * np.linalg.norm(u0)


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


@pytest.mark.parametrize("method", [0, 3, 4])
def test_warm_start_with_zero_rhs_column(native_lib, method):
    """A solve started from the caller's U (x0) whose second load case has a
    zero right-hand side returns the zero vector in that column (the column
    takes no iteration), and the first column as a cold solve does."""
    import torch
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(12, 6, 6)
    eng = _engine_for(tsk, mixed=method != 0)
    rho = torch.from_numpy(_rho(tsk.mesh.nelements, 31, lo=0.01)).to(_dev())
    eng.update(rho, 1.0, 1e-9, 3.0)
    f = torch.from_numpy(np.asarray(tsk.neumann_linear[0])).to(_dev())
    F = torch.stack([f, torch.zeros_like(f)], dim=1).contiguous()
    U = torch.from_numpy(np.random.default_rng(5).standard_normal((tsk.n_dof, 2))).to(_dev())
    comp, st = eng.solve(F, U, method, 1, 1e-10, 2000, 0.1, 50, x0=True)
    assert st.status == 0
    assert torch.count_nonzero(U[:, 1]).item() == 0
    assert comp[1] == 0.0
    U0 = torch.zeros((tsk.n_dof, 1), dtype=torch.float64, device=_dev())
    comp0, _ = eng.solve(f[:, None].contiguous(), U0, method, 1, 1e-10, 2000, 0.1, 50)
    assert abs(comp[0] - comp0[0]) <= 1e-9 * abs(comp0[0])


def test_status_nonfinite_density(native_lib):
    """A NaN density makes the solve end with TOPT_NONFINITE (a status code
    on the host; nothing faults)."""
    import torch
    from sktopt_gb300 import _native as N
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(12, 6, 6)
    for mixed, method in ((False, 0), (True, 4)):
        eng = _engine_for(tsk, mixed=mixed)
        r = _rho(tsk.mesh.nelements, 3, lo=0.01)
        r[17] = np.nan
        f = torch.from_numpy(np.asarray(tsk.neumann_linear[0])[:, None].copy()).to(_dev())
        U = torch.zeros_like(f)
        with pytest.raises(N.ToptError) as ei:
            eng.update(torch.from_numpy(r).to(_dev()), 1.0, 1e-9, 3.0)
            eng.solve(f, U, method, 1, 1e-8, 500, 0.1, 50)
        assert ei.value.code == N.TOPT_NONFINITE


def test_status_maxiter(native_lib):
    """maxiter = 1 on a 12x6x6 solve to 1e-8 ends with TOPT_MAXITER (reported,
    not raised, as the reference only logs CG non-convergence)."""
    import torch
    from sktopt_gb300 import _native as N
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(12, 6, 6)
    for mixed, method in ((False, 0), (True, 4)):
        eng = _engine_for(tsk, mixed=mixed)
        eng.update(torch.from_numpy(_rho(tsk.mesh.nelements, 4, lo=0.01)).to(_dev()),
                   1.0, 1e-9, 3.0)
        f = torch.from_numpy(np.asarray(tsk.neumann_linear[0])[:, None].copy()).to(_dev())
        U = torch.zeros_like(f)
        comp, st = eng.solve(f, U, method, 1, 1e-8, 1, 0.1, 1)
        assert st.status == N.TOPT_MAXITER, st
        assert np.isfinite(comp[0])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_elastic_plugin_numpy_call_convention(native_lib, precision):
    """FEM_SimpLinearElasticity at the reference's call convention
    (solver_elastic.py:643-676): NumPy rho in, u_dofs (n_dof, L) NumPy
    written in place, NumPy compliances and (n_elem, L) energies out; two
    load cases on a 10x5x4 cantilever against the oracle's direct solves."""
    from sktopt_gb300.fea.solver_elastic import FEM_SimpLinearElasticity, LinearSolverConfig
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(10, 5, 4)
    f0 = np.asarray(tsk.neumann_linear[0])
    f1 = np.zeros_like(f0)
    ijk = tsk.mesh.node_ijk
    top = np.nonzero((ijk[0] == 10) & (ijk[2] == 4))[0]
    f1[3 * top + 1] = 0.5 / top.size
    tsk.neumann_linear = [f0, f1]
    fem = FEM_SimpLinearElasticity(tsk, 1e-9, solver_config=LinearSolverConfig(
        solver="spsolve", precision=precision), device=_dev())
    rho = _rho(tsk.mesh.nelements, 41, lo=0.05)
    u_dofs = np.zeros((tsk.n_dof, 2))
    comp = fem.objectives_multi_load(rho, 3.0, u_dofs)
    assert isinstance(comp, np.ndarray) and comp.shape == (2,)
    en = fem.energy_multi_load(rho, 3.0, u_dofs)
    assert isinstance(en, np.ndarray) and en.shape == (tsk.mesh.nelements, 2)
    m, pb, *_ = problems.cantilever(10, 5, 4)
    pb.forces = [f0, f1]
    comp_ref, U_ref = pb.objectives(rho, 3.0, 1e-9, "spsolve")
    en_ref = pb.energy(rho, 3.0, 1e-9, U_ref)
    tol = 1e-10 if precision == "fp64" else 1e-6
    np.testing.assert_allclose(comp, comp_ref, rtol=tol)
    np.testing.assert_allclose(u_dofs, U_ref, rtol=0, atol=tol * np.abs(U_ref).max())
    assert np.linalg.norm(en - en_ref) <= (1e-9 if precision == "fp64" else 1e-5) * \
        np.linalg.norm(en_ref)
