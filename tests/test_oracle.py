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


# ------------------------------------------------------------------------------------------------
# Pinned to the reference's Material.cpp, SpinOrbitFunctional.cpp, Hamiltonian.cpp and
# BandStructure.cpp (compiled against oracle/shim's Eigen / yaml-cpp subsets; fixtures made by
# tests/golden/make_golden.py).

def _ref_fixture(name):
    return np.load(os.path.join(GOLDEN, name))


HAM_CASES = [("si_local", "si-cohen-bergstresser.yaml", "Si", 0, 0),
             ("si_nl", "materials.yaml", "Si", 1, 0),
             ("si_d", "si-nonlocal-d.yaml", "Si", 1, 0),
             ("inp_nl", "materials.yaml", "InP", 1, 0),
             ("ge_nl_soc", "materials.yaml", "Ge", 1, 1),
             ("gaas_nl_soc", "materials.yaml", "GaAs", 1, 1),
             ("gap_soc", "materials.yaml", "GaP", 0, 1)]


def test_material_loader_fields_equal_the_reference_loader(oracle):
    """Materials::load_material_parameters (Material.cpp:33-71, NonLocalParameters.hpp:91-116,
    SpinOrbitParameters.hpp:74-81): every field of every material of every params/ file."""
    from conftest import PARAMS

    ref = json.load(open(os.path.join(GOLDEN, "ref_materials.json")))
    assert ref
    for fname, mats in ref.items():
        got = oracle.load_materials(os.path.join(PARAMS, fname))
        assert set(got) == set(mats), fname
        for sym, fields in mats.items():
            for f, v in fields.items():
                assert getattr(got[sym], f) == v, (fname, sym, f)


@pytest.mark.parametrize("key,fname,sym,nl,soc", HAM_CASES)
def test_hamiltonian_bit_exact_with_reference_code(oracle, key, fname, sym, nl, soc):
    """H(k) after SetMatrix + Diagonalize's hermitisation (Hamiltonian.cpp:50-127), including the
    nonlocal correction (Material.cpp:87-208) and the spin-orbit blocks (SpinOrbitFunctional.cpp:
    20-138): every element bit-exact at basis 15, every matrix byte-identical (SHA-256) at the
    production bases (up to order 458), at Gamma, L, X, W, K, U and two generic k. Zeros compare
    unsigned: their sign follows how the matrix library scales a complex by a real in
    Diagonalize's 0.5 * (H + H^H), which the reference does not fix."""
    import hashlib

    from conftest import PARAMS

    d = _ref_fixture("ref_hamiltonian.npz")
    mat = oracle.load_materials(os.path.join(PARAMS, fname))[sym]
    G = d["G_small"]
    np.testing.assert_array_equal(G, oracle.generate_basis(3))
    n = (2 if soc else 1) * len(G)
    r, c = np.tril_indices(n)
    Gp = oracle.generate_basis(int(d[key + "_shells"]))
    for q, k in enumerate(d["k"]):
        H = oracle.assemble(mat, G, k, nl=bool(nl), soc=bool(soc))
        np.testing.assert_array_equal(H[r, c], d[key + "_lower"][q])
        Hp = oracle.assemble(mat, Gp, k, nl=bool(nl), soc=bool(soc))
        assert hashlib.sha256((Hp + 0.0).tobytes(order="F")).hexdigest() == str(d[key + "_sha256"][q]), (key, q)


@pytest.mark.parametrize("key,fname,sym,nl,soc", [c for c in HAM_CASES if c[3] or c[4]])
def test_nonlocal_and_spin_orbit_elements_bit_exact(oracle, key, fname, sym, nl, soc):
    """Material::compute_pseudopotential_non_local_correction and
    SpinOrbitCorrection::compute_soc_contribution on seeded pairs, with the |K1| = |K2| branches of
    F_l (equal vectors, signed permutations) and K = 0."""
    import ctypes as C

    from conftest import PARAMS

    d = _ref_fixture("ref_elements.npz")
    L = oracle.lib()
    mat = oracle.load_materials(os.path.join(PARAMS, fname))[sym]
    tau = np.full(3, (1.0 / 8.0) * 1e-10 * mat.lattice_constant)
    out2, out8 = np.zeros(2), np.zeros(8)
    dp = oracle._dp
    for q in range(len(d["K1"])):
        K1, K2 = np.ascontiguousarray(d["K1"][q]), np.ascontiguousarray(d["K2"][q])
        if nl:
            L.or_nl_correction(C.byref(mat), dp(K1), dp(K2), dp(tau), dp(out2))
            np.testing.assert_array_equal(out2, d[key + "_nl"][q], err_msg=f"{key} nl pair {q}")
        if soc:
            G1, G2 = np.ascontiguousarray(d["G1"][q]), np.ascontiguousarray(d["G2"][q])
            assert L.or_soc_block(C.byref(mat), dp(K1), dp(K2), dp(G1), dp(G2), dp(tau), dp(out8)) == 0
            np.testing.assert_array_equal(out8, d[key + "_soc"][q], err_msg=f"{key} soc pair {q}")


def test_band_structure_energies_equal_the_reference_code(oracle):
    """BandStructure::Initialize (path) + Compute + AdjustValues of the reference against the
    oracle's band structure and AdjustValues on the same path (the solver is shared, so this pins
    the assembly, the band count after the SOC doubling and AdjustValues)."""
    from conftest import PARAMS

    d = _ref_fixture("ref_bands.npz")
    cases = [("si_local", "si-cohen-bergstresser.yaml", "Si", 16, "LGXWKULWXKG", 40, 10, 0, 0),
             ("ge_nl_soc", "materials.yaml", "Ge", 8, "LGX", 20, 8, 1, 1)]
    for key, fname, sym, nb, labels, npts, shells, nl, soc in cases:
        mat = oracle.load_materials(os.path.join(PARAMS, fname))[sym]
        k, _ = oracle.generate_path(labels, npts)
        nbt = nb * (2 if soc else 1)
        r = oracle.band_structure(mat, oracle.generate_basis(shells), k, nbt, nl=bool(nl), soc=bool(soc), nthreads=1)
        E = np.ascontiguousarray(r["E"])
        oracle.adjust_values(E, soc=bool(soc), min_cond_zero=False)
        np.testing.assert_array_equal(E, d[key])


def test_gradient_array_shape_of_the_reference():
    """Compute_parallel(true, n) sizes m_energies_gradient as [nk * nb] rows of nb
    (BandStructure.cpp:158-166) and fills only the first nk rows."""
    d = _ref_fixture("ref_gradients.npz")
    nk, nb = len(d["k"]), int(d["nb"])
    assert int(d["rows"]) == nk * nb and int(d["row_len"]) == nb


def test_gradients_equal_the_reference_code(oracle):
    """compute_gradient_at_level (Hamiltonian.cpp:146-194) of the reference against the oracle's."""
    from conftest import PARAMS

    d = _ref_fixture("ref_gradients.npz")
    mat = oracle.load_materials(os.path.join(PARAMS, "si-cohen-bergstresser.yaml"))["Si"]
    r = oracle.band_structure(mat, d["G"], d["k"], int(d["nb"]), grad=True, nthreads=1)
    np.testing.assert_array_equal(r["grad"], d["grad"])


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "libref.so")),
                    reason="reference checker library not built (reference tree absent)")
def test_hamiltonian_live_against_reference_code_on_random_k(oracle):
    """Where the reference tree is present: the reference's own Hamiltonian on 24 seeded k per case
    at basis 27, element-wise bit-exact with the oracle."""
    from conftest import PARAMS

    R = oracle.ref_lib()
    if R is None:
        pytest.skip("reference checker library not built")
    G = oracle.generate_basis(4)
    k = np.random.default_rng(7).uniform(-1.0, 1.0, (24, 3))
    for key, fname, sym, nl, soc in HAM_CASES:
        path = os.path.join(PARAMS, fname)
        n = (2 if soc else 1) * len(G)
        H = np.zeros((len(k), n, n), dtype=np.complex128)
        assert R.ref_hamiltonian(path.encode(), sym.encode(), oracle._ip(G), len(G), oracle._dp(k), len(k), nl, soc,
                                 oracle._dp(H)) == n
        mat = oracle.load_materials(path)[sym]
        for q in range(len(k)):
            np.testing.assert_array_equal(oracle.assemble(mat, G, k[q], nl=bool(nl), soc=bool(soc)), H[q].T,
                                          err_msg=f"{key} k {q}")
