"""The oracle pinned against the reference: its own golden tables, its own code compiled here
(fixtures from oracle/_ref), LAPACK for the restated Eigen solver, and physics known answers.
CPU only."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.filterwarnings("ignore")


def test_bessel_golden_table_of_the_reference(oracle):
    """tests/epp/test_bessel_functions.cpp:22-65 with doctest::Approx's default tolerance."""
    L = oracle.lib()
    t = json.load(open(os.path.join(GOLDEN, "bessel_table.json")))
    nx = len(t["list_x"])
    for i, nu in enumerate(t["list_nu"]):
        for j, x in enumerate(t["list_x"]):
            want_c = t["nu_x_bessel_cyl_values"][i * nx + j]
            want_s = t["nu_x_bessel_values"][i * nx + j]
            got_c = L.or_cyl_bessel(nu, x)
            got_s = L.or_sph_bessel(nu, x)
            # doctest::Approx: |a-b| < eps * (scale + max(|a|,|b|)), eps = float epsilon * 100
            eps = np.finfo(np.float32).eps * 100
            assert abs(got_c - want_c) < eps * (1 + max(abs(got_c), abs(want_c))), (nu, x, got_c, want_c)
            assert abs(got_s - want_s) < eps * (1 + max(abs(got_s), abs(want_s))), (nu, x, got_s, want_s)


def test_bessel_bit_exact_with_reference_code(oracle):
    L = oracle.lib()
    d = np.load(os.path.join(GOLDEN, "ref_bessel.npz"))
    for a, nu in enumerate(d["nu"]):
        got = np.array([L.or_sph_bessel(nu, x) for x in d["x"]])
        np.testing.assert_array_equal(got, d["sph"][a])
    for a, nu in enumerate(d["cyl_nu"]):
        got = np.array([L.or_cyl_bessel(nu, x) for x in d["cyl_x"]])
        np.testing.assert_array_equal(got, d["cyl"][a])
    got = np.array([L.or_bessel_i2(x) for x in d["i2_x"]])
    np.testing.assert_array_equal(got, d["i2"])


def test_local_form_factor_bit_exact_with_reference_code(oracle):
    import ctypes as C

    L = oracle.lib()
    d = np.load(os.path.join(GOLDEN, "ref_pp.npz"))
    for key in ("si_cb", "gaas_pv"):
        V = d[key + "_V"]
        m = oracle.OrMaterial()
        m.V3S, m.V4S, m.V8S, m.V11S, m.V3A, m.V4A, m.V8A, m.V11A = V
        a = float(d[key + "_a"])
        tau = np.full(3, (1.0 / 8.0) * a)
        out = np.zeros(2)
        got = np.zeros_like(d[key])
        for q, (x, y, z) in enumerate(d["dG"]):
            L.or_pp_value(C.byref(m), int(x), int(y), int(z), oracle._dp(tau), a, oracle._dp(out))
            got[q] = out
        np.testing.assert_array_equal(got, d[key])


def test_path_bit_exact_with_reference_code(oracle):
    for e in json.load(open(os.path.join(GOLDEN, "ref_paths.json"))):
        if e["count"] < 0:
            with pytest.raises(ValueError):
                oracle.generate_path(e["labels"], e["n"])
            continue
        k, pos = oracle.generate_path(e["labels"], e["n"])
        np.testing.assert_array_equal(k.ravel(), np.array(e["k"]))
        assert pos == e["sym"]


@pytest.mark.parametrize("shells,size", [(2, 9), (3, 15), (4, 27), (8, 89), (9, 113), (10, 137), (11, 169),
                                         (12, 181), (13, 229)])
def test_basis_sizes(oracle, shells, size):
    G = oracle.generate_basis(shells)
    assert G.shape == (size, 3)
    g2 = (G * G).sum(1)
    assert g2.max() <= oracle.lib().or_shell_table_size() * 10
    assert tuple(G[len(G) // 2]) == (0, 0, 0)  # i -> j -> k loop order puts G = 0 in the middle


def test_basis_rejects_bad_shell_counts(oracle):
    with pytest.raises(RuntimeError):
        oracle.generate_basis(1)
    with pytest.raises(RuntimeError):
        oracle.generate_basis(200)


def test_restated_eigen_solver_against_lapack(oracle):
    rng = np.random.default_rng(7)
    for n in (1, 2, 5, 33, 90):
        A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        A = A + A.conj().T
        w, Z = oracle.eigh(A, vectors=True)
        wl = np.linalg.eigvalsh(A)
        np.testing.assert_allclose(w, wl, atol=1e-12 * max(1, np.abs(wl).max()))
        np.testing.assert_allclose(A @ Z, Z * w, atol=1e-11 * max(1, np.abs(wl).max()))
        np.testing.assert_allclose(Z.conj().T @ Z, np.eye(n), atol=1e-12)


def test_restated_eigen_solver_degenerate(oracle):
    # exactly repeated eigenvalues (the Gamma-point triplets of the diamond structure)
    rng = np.random.default_rng(3)
    Q, _ = np.linalg.qr(rng.normal(size=(12, 12)) + 1j * rng.normal(size=(12, 12)))
    d = np.array([1, 1, 1, 2, 2, 3, 4, 4, 4, 4, 5, 6], float)
    A = (Q * d) @ Q.conj().T
    A = 0.5 * (A + A.conj().T)
    w = oracle.eigh(A)
    np.testing.assert_allclose(w, d, atol=1e-13)


def test_hamiltonian_is_hermitian(oracle, mats):
    for name, nl, soc in [("Si-CB", 0, 0), ("Si-d", 1, 0), ("Ge", 1, 1), ("GaAs", 1, 1), ("InP", 1, 0)]:
        G = oracle.generate_basis(8)
        H = oracle.assemble(mats[name], G, [0.13, -0.27, 0.41], nl=nl, soc=soc)
        assert np.array_equal(H, H.conj().T)


def test_free_electron_limit(oracle):
    """All form factors zero: H is diagonal with C |k+G|^2, C = hbar^2/(2 m q) (2 pi / a)^2."""
    m = oracle.OrMaterial()
    m.lattice_constant = 5.43
    G = oracle.generate_basis(10)
    k = np.array([0.1, 0.2, 0.3])
    E = oracle.band_structure(m, G, k[None], 20)["E"][0]
    a = 5.43e-10
    C = oracle.H_BAR ** 2 / (2 * oracle.M_E * oracle.Q_E) * (2 * np.pi / a) ** 2
    want = np.sort(C * ((k + G) ** 2).sum(1))[:20]
    np.testing.assert_allclose(E, want, rtol=1e-13)


def test_si_gamma_point_degeneracies(oracle, mats):
    G = oracle.generate_basis(10)
    E = oracle.band_structure(mats["Si-CB"], G, np.zeros((1, 3)), 8)["E"][0]
    # Gamma_25' valence triplet and Gamma_15 conduction triplet
    assert np.ptp(E[1:4]) < 1e-12 and np.ptp(E[4:7]) < 1e-12
    assert 3.2 < E[4] - E[3] < 3.6  # the well-known ~3.4 eV direct gap of this form-factor set


def test_kramers_pairs_with_soc(oracle, mats):
    # Ge has inversion symmetry: with SOC every band is doubly degenerate at every k
    G = oracle.generate_basis(8)
    k = oracle.sample_first_bz(3, 11)
    E = oracle.band_structure(mats["Ge"], G, k, 16, nl=True, soc=True)["E"]
    np.testing.assert_allclose(E[:, 0::2], E[:, 1::2], atol=1e-9)
    # At Gamma the p-like triplet splits into a quartet above a split-off pair. The reference's SOC
    # term uses the reduced K x K' without the kfac^2 its comment mentions
    # (SpinOrbitFunctional.cpp:129-135), so the splitting is ~0.015 eV rather than Ge's measured
    # 0.29 eV; the oracle reproduces the reference, not the measurement.
    E0 = oracle.band_structure(mats["Ge"], G, np.zeros((1, 3)), 8, nl=True, soc=True)["E"][0]
    assert np.ptp(E0[4:8]) < 1e-9 and np.ptp(E0[2:4]) < 1e-9
    assert 0.005 < E0[4] - E0[2] < 0.05


def test_cubic_symmetry_of_bands(oracle, mats):
    """E(k) = E(Sk) for cubic point-group operations (permutations and sign changes of k)."""
    G = oracle.generate_basis(9)
    k = np.array([[0.12, 0.31, -0.07]])
    ops = [k[:, [1, 0, 2]], k[:, [2, 1, 0]], -k, k * np.array([1, -1, 1]), k[:, [1, 2, 0]] * np.array([-1, 1, -1])]
    for name, nl in [("Si-CB", 0), ("Si-d", 1), ("Ge", 1)]:
        E0 = oracle.band_structure(mats[name], G, k, 12, nl=nl)["E"]
        for kk in ops:
            E1 = oracle.band_structure(mats[name], G, kk, 12, nl=nl)["E"]
            np.testing.assert_allclose(E1, E0, atol=1e-11)


def test_gradient_matches_finite_difference(oracle, mats):
    """The Hellmann-Feynman kinetic gradient equals dE/dk for a local Hamiltonian (non-degenerate)."""
    G = oracle.generate_basis(9)
    k = np.array([0.21, 0.13, 0.05])
    r = oracle.band_structure(mats["Si-CB"], G, k[None], 6, grad=True)
    a = 5.43e-10
    h = 1e-6
    for c in range(3):
        dk = np.zeros(3)
        dk[c] = h
        Ep = oracle.band_structure(mats["Si-CB"], G, (k + dk)[None], 6)["E"][0]
        Em = oracle.band_structure(mats["Si-CB"], G, (k - dk)[None], 6)["E"][0]
        fd = (Ep - Em) / (2 * h) / (2 * np.pi / a)  # eV per (1/m)
        np.testing.assert_allclose(r["grad"][0, :, c], fd, rtol=1e-5, atol=1e-16)


def test_adjust_values_matches_reference_semantics(oracle):
    E = np.array([[-1.0, 0.0, 0.5, 1.0, 2.0, 3.0], [-1.2, 0.1, 0.6, 0.9, 2.2, 3.5]])
    gap, found = oracle.adjust_values(E)
    assert found and gap == pytest.approx(2.0 - 1.0)
    assert E[0, 3] == pytest.approx(0.0) and E[0, 4] == pytest.approx(1.0)


def test_unsupported_soc_period_is_rejected(oracle, mats):
    G = oracle.generate_basis(4)
    with pytest.raises(RuntimeError):
        oracle.assemble(mats["Sn"], G, [0.1, 0.0, 0.0], soc=True)  # Sn has atomic period 5


def _isolated(E, tol=1e-3):
    """Bands separated from both neighbours by more than tol eV, the top band excluded (its upper
    neighbour is not in the fixture): their gradients are well defined."""
    gaps = np.diff(E)
    iso = (np.r_[np.inf, gaps] > tol) & (np.r_[gaps, 0.0] > tol)
    return iso


def test_oracle_reproduces_its_band_fixtures(oracle):
    """tests/golden/oracle_bands.npz (make_oracle_golden.py): eigenvalues and, for isolated bands,
    Hellmann-Feynman gradients at the symmetry points and two seeded k, for five configurations."""
    import sys

    sys.path.insert(0, GOLDEN)
    import make_oracle_golden as MG

    fx = np.load(os.path.join(GOLDEN, "oracle_bands.npz"))
    np.testing.assert_array_equal(fx["k"], MG.k_points())
    for name in MG.CONFIGS:
        E, g = MG.compute(name)
        np.testing.assert_allclose(E, fx[name + "_E"], rtol=0, atol=1e-10, err_msg=name)
        scale = np.abs(fx[name + "_grad"]).max()
        for q in range(len(E)):
            iso = _isolated(fx[name + "_E"][q])
            np.testing.assert_allclose(g[q][iso], fx[name + "_grad"][q][iso], rtol=0, atol=1e-8 * scale, err_msg=name)
