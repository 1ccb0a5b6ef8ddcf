"""Band states over a BZ mesh and their dielectric function (BZ_States, src/BZ_MESH/bz_states.cpp):
the MSH tetrahedron reader, tetrahedron volumes and per-vertex weights on the CPU; on the GPU the
mesh dielectric function (device eigenstates at every vertex at k and k + q, one weighted pass of
the overlap sums) against the oracle's tetrahedron loop."""
import math
import os

import numpy as np
import pytest

from ultimateepm_gb300 import _native as N
from ultimateepm_gb300 import api
from ultimateepm_gb300 import mesh as M
from ultimateepm_gb300.bz_states import BZ_States

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PARAMS = os.path.join(ROOT, "params")


def _cube_mesh(n=3, lo=0.07, step=0.11):
    """Vertices of an n x n x n grid (reduced k, generic offset) and each cube cut into 6 tetrahedra."""
    idx = lambda i, j, k: (i * n + j) * n + k
    pts = np.array([[lo + step * i + 0.013 * j, lo + step * j, lo + step * k + 0.007 * i]
                    for i in range(n) for j in range(n) for k in range(n)])
    tets = []
    for i in range(n - 1):
        for j in range(n - 1):
            for k in range(n - 1):
                c = [idx(i + a, j + b, k + d) for a in (0, 1) for b in (0, 1) for d in (0, 1)]
                v0, v7 = c[0], c[7]
                for a, b in ((1, 3), (3, 2), (2, 6), (6, 4), (4, 5), (5, 1)):
                    tets.append([v0, c[a], c[b], v7])
    return pts, np.array(tets, dtype=np.int64)


def _write_msh(path, pts, tets, version):
    with open(path, "w") as f:
        if version == 4:
            f.write("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n")
            f.write(f"$Nodes\n1 {len(pts)} 1 {len(pts)}\n3 1 0 {len(pts)}\n")
            for q in range(len(pts)):
                f.write(f"{q + 1}\n")
            for p in pts:
                f.write(" ".join(repr(float(x)) for x in p) + "\n")
            f.write("$EndNodes\n")
            f.write(f"$Elements\n2 {len(tets) + 1} 1 {len(tets) + 1}\n")
            f.write("2 1 2 1\n1 1 2 3\n")  # a triangle block, skipped
            f.write(f"3 1 4 {len(tets)}\n")
            for q, t in enumerate(tets):
                f.write(f"{q + 2} " + " ".join(str(int(x) + 1) for x in t) + "\n")
            f.write("$EndElements\n")
        else:
            f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n")
            f.write(f"$Nodes\n{len(pts)}\n")
            for q, p in enumerate(pts):
                f.write(f"{q + 1} " + " ".join(repr(float(x)) for x in p) + "\n")
            f.write("$EndNodes\n")
            f.write(f"$Elements\n{len(tets) + 1}\n")
            f.write("1 2 2 0 1 1 2 3\n")
            for q, t in enumerate(tets):
                f.write(f"{q + 2} 4 2 0 1 " + " ".join(str(int(x) + 1) for x in t) + "\n")
            f.write("$EndElements\n")


@pytest.mark.parametrize("version", [4, 2])
def test_msh_tetrahedra_and_weights(tmp_path, version):
    pts, tets = _cube_mesh(3)
    path = str(tmp_path / f"m{version}.msh")
    _write_msh(path, pts, tets, version)
    np.testing.assert_array_equal(M.read_msh_tetrahedra(path), tets + 1)
    mats = api.Materials()
    mats.load_material_parameters(os.path.join(PARAMS, "si-cohen-bergstresser.yaml"))
    st = BZ_States(mats.materials["Si"])
    st.read_mesh_geometry_from_msh_file(path, False)
    assert st.tetra.shape == tets.shape
    vol = M.tetra_signed_volumes(pts, tets)
    np.testing.assert_allclose(st.tetra_volumes, vol, rtol=1e-15)
    assert np.all(np.abs(vol) > 0)
    w = st.vertex_weights()
    np.testing.assert_allclose(w.sum(), np.abs(vol).sum(), rtol=1e-14)
    # a degenerate tetrahedron (|V| < 1e-12) is dropped
    st.set_tetrahedra(np.vstack([tets, [[0, 1, 2, 2]]]))
    assert len(st.tetra) == len(tets)
    with pytest.raises(ValueError):
        st.set_tetrahedra([[0, 1, 2, len(pts)]])


@pytest.mark.gpu
def test_mesh_dielectric_function_matches_the_oracle(gpu, oracle, mats, tmp_path):
    pts, tets = _cube_mesh(3)
    si = api.Material("Si", raw=N.UepmMaterial.from_buffer_copy(bytes(mats["Si-CB"])))
    a = si.get_lattice_constant_meter()
    G = oracle.generate_basis(9)
    nb = 10
    st = BZ_States(si)
    st.set_vertices(pts)
    st.set_tetrahedra(tets)
    st.set_nb_bands(nb)
    st.set_basis_vectors(G)
    st.compute_eigenstates()
    q = np.array([0.02, 0.01, -0.015])
    st.compute_shifted_eigenstates(q)
    en = np.linspace(0.0, 8.0, 160)
    st.compute_dielectric_function(en, 0.08)
    got = st.m_dielectric_function_real
    ok = oracle.band_structure(mats["Si-CB"], G, pts, nb, vectors=True)
    okq = oracle.band_structure(mats["Si-CB"], G, pts + q, nb, vectors=True)
    vol = M.tetra_signed_volumes(pts * (2 * math.pi / a), tets)
    ref = oracle.bz_states_dielectric(ok["E"], ok["vecs"], okq["E"], okq["vecs"], tets, vol, en, 0.08,
                                      q * (2 * math.pi / a))
    np.testing.assert_allclose(got - 1.0, ref - 1.0, rtol=1e-9, atol=1e-9 * np.abs(ref - 1.0).max())
    path = str(tmp_path / "si")
    st.export_dielectric_function(path)
    assert open(path + "_dielectric_function.csv").readline().strip() == "Energy (eV),Dielectric function"
