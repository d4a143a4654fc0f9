"""Kohn-Sham pieces: the potential matrix (build_mass_V_matrix,
src/Discretize.cpp:668-843) against the oracle, quadrature-point values of FE
functions, densities, matrix addition, and helium SCFs (one pinned to the oracle's
Kohn-Sham loop)."""
import os

import numpy as np
import pytest
import scipy.sparse as sps

import oracle
from tsemlib_gb300 import ks, mesh, tsem

pytestmark = pytest.mark.gpu


def _sp(A):
    rp, c, v = A.arrays()
    n = len(rp) - 1
    return sps.csr_matrix((v, c, rp), shape=(n, n))


def _space(n=2, p=4, jitter=0.1, shuffle=False):
    m = mesh.kuhn_cube(n, jitter, 3)
    if shuffle:
        m = mesh.shuffle_local_order(m, 4)
    return mesh.mark_all_boundary(m)


@pytest.mark.parametrize("shuffle", [False, True])
def test_potential_matrix_matches_oracle(shuffle):
    m = _space(shuffle=shuffle)
    T = tsem.TSEM(4, 6, m)
    S = oracle.Space(m, 4, quad_q=6)
    rng = np.random.default_rng(1)
    v = rng.uniform(-2.0, 3.0, (T.n_element, T.n_q_point[2]))
    A = _sp(T.build_mass_V_matrix(v))
    B = _sp(S.assemble_potential(v))
    assert abs(A - B).max() <= 1e-13 * abs(B).max()
    # rows keep the diagonal first
    rp, c, _ = T.build_mass_V_matrix(v).arrays()
    assert np.array_equal(c[rp[:-1]], np.arange(len(rp) - 1))


def test_unit_potential_is_the_mass_matrix_and_refill_in_place():
    """V = 1 gives the mass matrix.  The potential matrix is summed with split FP32
    operands (about 2^-44 relative per entry), so the bar is the 1e-13 relative bar of
    the assembled matrices, not FP64 rounding."""
    m = _space()
    T = tsem.TSEM(4, 6, m)
    one = np.ones((T.n_element, T.n_q_point[2]))
    MV = T.build_mass_V_matrix(one)
    assert abs(_sp(MV) - _sp(T.mass_matrix)).max() <= 1e-13 * abs(_sp(T.mass_matrix)).max()
    again = T.build_mass_V_matrix(2.0 * one, out=MV)
    assert again is MV
    assert abs(_sp(MV) - 2.0 * _sp(T.mass_matrix)).max() <= 1e-13 * abs(_sp(T.mass_matrix)).max()


def test_quadrature_values_integrate_like_the_matrices():
    m = _space()
    T = tsem.TSEM(4, 6, m)
    x = np.random.default_rng(2).standard_normal(T.n_dof_total)
    W = T.geometry()["volume"][:, None] * T.quadrature()["w3"][None, :]
    u = T.value_qp(x)
    ones = T.calc_rhs(value_f=np.ones_like(u))
    assert np.sum(W * u) == pytest.approx(ones @ x, rel=1e-12)
    assert np.sum(W * u * u) == pytest.approx(x @ T.mass_matrix.vmult(x), rel=1e-12)


@pytest.mark.parametrize("shuffle", [False, True])
def test_density_matches_oracle(shuffle):
    """calc_density and calc_density_l2_difference against the oracle's restatement
    (src/PointInfo.cpp:72-91, src/CalcError.cpp:703-735); the device-array form gives
    the host form's values bit for bit."""
    torch = pytest.importorskip("torch")
    m = _space(shuffle=shuffle)
    T = tsem.TSEM(4, 6, m)
    S = oracle.Space(m, 4, quad_q=6)
    rng = np.random.default_rng(8)
    psi = rng.standard_normal((3, T.n_dof_total))
    occ = [2.0, 1.0, 0.5]
    rho = T.calc_density(psi, occ)
    ref = S.density(psi, occ)
    assert np.abs(rho - ref).max() <= 1e-13 * np.abs(ref).max()
    pd = torch.from_numpy(psi).cuda()
    out = torch.empty(rho.shape, dtype=torch.float64, device="cuda")
    T.calc_density_device(pd.data_ptr(), occ, out.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), rho)
    phi = psi + 1e-3 * rng.standard_normal(psi.shape)
    d = T.calc_density_l2_difference(psi, phi, occ)
    d_o = S.density_l2_difference(psi, phi, occ)
    assert d == pytest.approx(d_o, rel=1e-12)
    assert T.calc_density_l2_difference(psi, psi, occ) == 0.0
    with pytest.raises(tsem.TsemError):
        T.calc_density(np.zeros((65, T.n_dof_total)), np.ones(65))


def test_matrix_add():
    m = _space()
    T = tsem.TSEM(4, 6, m)
    v = np.random.default_rng(3).uniform(0.5, 1.5, (T.n_element, T.n_q_point[2]))
    H = T.build_mass_V_matrix(v)
    ref = _sp(H) + 0.5 * _sp(T.stiff_matrix)
    H.add(0.5, T.stiff_matrix)
    assert abs(_sp(H) - ref).max() <= 1e-14 * abs(ref).max()
    with pytest.raises(tsem.TsemError):
        T.stiff_matrix.copy().add(1.0, H)       # H's pattern is larger than the stiffness pattern


def test_helium_scf_converges():
    out = ks.helium(p=3, n_half=3, max_iter=40, tol=1e-8)
    assert out["converged"], out["history"][-3:]
    h = out["history"][-1]
    assert h["charge"] == pytest.approx(2.0, abs=1e-6)
    # exchange-only LDA helium is about -2.72 Hartree; a coarse mesh is a little above it
    assert -3.0 < out["energy"] < -2.3
    ev = out["eigenvalues"]
    assert ev[0] < 0 and all(a <= b + 1e-12 for a, b in zip(ev, ev[1:]))


def test_helium_energy_matches_oracle():
    """Same mesh, order and physics as the oracle's FP64 Kohn-Sham loop
    (tests/ks_oracle.py, fixture from tests/golden/make_helium_energy.py): the
    self-consistent energies agree to the SCF tolerance.  The energy is stationary in
    the density, so it pins to 1e-7; the eigenvalues move with the density itself
    and pin to 1e-4."""
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "helium_graded2_p4.npz"))
    out = ks.helium(p=int(ref["p"]), n_half=int(ref["n_half"]), ratio=float(ref["ratio"]),
                    half_width=float(ref["half_width"]), max_iter=60, tol=1e-10, eig_tol=1e-10)
    assert out["converged"], out["history"][-3:]
    assert abs(out["energy"] - float(ref["energy"])) <= 1e-7
    assert np.abs(np.asarray(out["eigenvalues"][:4]) - ref["eigenvalues"]).max() <= 1e-4


def test_device_array_forms_match_host_forms():
    """value_qp / calc_rhs / build_mass_V_matrix on device arrays give the host forms' results."""
    torch = pytest.importorskip("torch")
    m = _space(shuffle=True)
    T = tsem.TSEM(4, 6, m)
    rng = np.random.default_rng(4)
    x = rng.standard_normal(T.n_dof_total)
    v = rng.uniform(-1.0, 2.0, (T.n_element, T.n_q_point[2]))
    xd = torch.from_numpy(x).cuda()
    vd = torch.from_numpy(v).cuda()
    uq = torch.empty_like(vd)
    T.value_qp_device(xd.data_ptr(), uq.data_ptr())
    bd = torch.empty_like(xd)
    T.calc_rhs_device(vd.data_ptr(), bd.data_ptr())
    Hd = T.build_mass_V_matrix_device(vd.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(uq.cpu().numpy(), T.value_qp(x))
    assert np.abs(bd.cpu().numpy() - T.calc_rhs(value_f=v)).max() <= 1e-13 * np.abs(T.calc_rhs(value_f=v)).max()
    H = T.build_mass_V_matrix(v)
    assert abs(_sp(Hd) - _sp(H)).max() <= 1e-13 * abs(_sp(H)).max()
