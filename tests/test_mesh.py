"""Band structure over a Brillouin-zone mesh (ultimateepm_gb300.mesh): the MSH node reader, the
irreducible-wedge test and the signed-permutation rule against the oracle's restatement of the
reference (MeshBZ::is_irreducible_wedge, apply_same_symmetry_operation), the k-star of a symmetric
vertex set, the reference's kstar file format, the host and device wedge -> full-zone distribution,
and (GPU) energies and gradients at every vertex against direct solves."""
import ctypes as C
import itertools
import os

import numpy as np
import pytest

from conftest import PARAMS, REFERENCE_ROOT
from ultimateepm_gb300 import _native as N
from ultimateepm_gb300 import api
from ultimateepm_gb300.mesh import MeshBZ, read_msh_nodes

REF_MESH = os.path.join(REFERENCE_ROOT, "examples", "meshes", "bz_mesh.msh")


def _si():
    mats = api.Materials()
    mats.load_material_parameters(os.path.join(PARAMS, "si-cohen-bergstresser.yaml"))
    return mats.materials["Si"]


def _cubic_group():
    ops = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            ops.append((perm, signs))
    return ops  # 48 signed permutations


def _star_set(nw, seed, extra_special=True):
    """Random wedge points (plus points with equal / zero components) and all their cubic images."""
    rng = np.random.default_rng(seed)
    pts = []
    while len(pts) < nw:
        x, y, z = np.sort(rng.uniform(0.0, 1.0, 3))[::-1]
        if x + y + z <= 1.5:
            pts.append((x, y, z))
    if extra_special:
        pts += [(0.5, 0.5, 0.0), (0.3, 0.2, 0.2), (0.0, 0.0, 0.0), (0.4, 0.0, 0.0), (0.25, 0.25, 0.25)]
    out = set()
    for p in pts:
        for perm, signs in _cubic_group():
            out.add(tuple(round(signs[j] * p[perm[j]], 12) + 0.0 for j in range(3)))
    arr = np.array(sorted(out))
    rng.shuffle(arr)
    return arr


def test_read_msh_41_and_22(tmp_path):
    p41 = tmp_path / "m41.msh"
    p41.write_text("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n$Nodes\n2 3 1 3\n0 1 0 1\n1\n0.5 0.25 0\n"
                   "3 1 0 2\n2\n3\n-0.5 0.1 0.2\n0.3 -0.3 0.1\n$EndNodes\n")
    tags, xyz = read_msh_nodes(str(p41))
    assert list(tags) == [1, 2, 3]
    np.testing.assert_array_equal(xyz, [[0.5, 0.25, 0], [-0.5, 0.1, 0.2], [0.3, -0.3, 0.1]])
    p22 = tmp_path / "m22.msh"
    p22.write_text("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n2\n1 0.1 0.2 0.3\n2 -1 0 1\n$EndNodes\n")
    tags, xyz = read_msh_nodes(str(p22))
    assert list(tags) == [1, 2] and xyz[1, 0] == -1.0
    pb = tmp_path / "bin.msh"
    pb.write_text("$MeshFormat\n4.1 1 8\n$EndMeshFormat\n")
    with pytest.raises(ValueError):
        read_msh_nodes(str(pb))


@pytest.mark.skipif(not os.path.exists(REF_MESH), reason="reference tree not present")
def test_reads_the_reference_mesh():
    tags, xyz = read_msh_nodes(REF_MESH)
    assert len(tags) == 14705 and xyz.shape == (14705, 3)
    assert (tags == np.arange(1, 14706)).all()
    m = MeshBZ(_si()).read_mesh_geometry_from_msh_file(REF_MESH, True)
    assert m.is_irreducible_wedge(m.positions).sum() > 0


def test_wedge_test_matches_the_oracle(oracle):
    rng = np.random.default_rng(2)
    k = rng.uniform(-1.1, 1.1, size=(3000, 3))
    k[:500] = np.sort(np.abs(k[:500]), axis=1)[:, ::-1]  # many inside
    m = MeshBZ(_si()).set_vertices(k)
    got = m.is_irreducible_wedge(m.positions)
    ref = np.array([oracle.is_irreducible_wedge(q) for q in m.reduced()])
    assert (got == ref).all() and got.sum() > 100


def test_signed_permutations_match_the_oracle(native, oracle):
    pts = _star_set(6, 3)
    rng = np.random.default_rng(4)
    a = pts[rng.integers(0, len(pts), 400)]
    ops = _cubic_group()
    b = np.array([[s[j] * q[p[j]] for j in range(3)] for q, (p, s) in zip(a, [ops[i] for i in rng.integers(0, 48, 400)])])
    b[:5] = [0.7, 0.1, 0.05]  # not a signed permutation of a
    op = np.zeros(len(a), dtype=np.uint16)
    found = np.zeros(len(a), dtype=np.int32)
    dp = lambda x: np.ascontiguousarray(x).ctypes.data_as(C.POINTER(C.c_double))
    N.check(native.uepm_star_operations(dp(a), dp(b), len(a), op.ctypes.data_as(C.POINTER(C.c_uint16)),
                                        found.ctypes.data_as(C.POINTER(C.c_int32))))
    for q in range(len(a)):
        ok, perm, sign = oracle.symmetry_operation(a[q], b[q])
        assert bool(found[q]) == ok
        assert [(op[q] >> (2 * j)) & 3 for j in range(3)] == perm
        assert [-1 if (op[q] >> (6 + j)) & 1 else 1 for j in range(3)] == sign


def test_kstar_of_a_symmetric_set_and_the_reference_file_format(native, tmp_path):
    k = _star_set(5, 9)
    m = MeshBZ(_si()).set_vertices(k).build_kstar_ibz_to_bz()
    kr = m.reduced()
    folded = -np.sort(-np.abs(kr), axis=1)
    np.testing.assert_allclose(folded, folded[m.src], atol=1e-9)
    assert sum(len(v) for v in m.kstar.values()) == len(k)
    assert all(m.is_irreducible_wedge(m.positions[m.iw_vertices]))
    assert m.ops_found.all()
    # the reference's kstar file, written and read back
    f = tmp_path / "mesh_kstar_ibz_to_bz.txt"
    with open(f, "w") as out:
        out.write("# iw m ids\n")
        for iw, ids in m.kstar.items():
            out.write(f"{iw} {len(ids)} " + " ".join(map(str, ids)) + "\n")
    m2 = MeshBZ(_si()).set_vertices(k).load_kstar_ibz_to_bz(str(f))
    assert (m2.src == m.src).all() and (m2.ops == m.ops).all()


def test_host_distribution_follows_the_reference_rule(native, oracle):
    k = _star_set(4, 12)
    m = MeshBZ(_si()).set_vertices(k).build_kstar_ibz_to_bz()
    rng = np.random.default_rng(1)
    used = np.asarray(m.iw_vertices)
    E_iw = rng.normal(size=(len(used), 6))
    g_iw = rng.normal(size=(len(used), 6, 3))
    pos = np.full(len(k), -1)
    pos[used] = np.arange(len(used))
    E, g = m.distribute_energies_from_iw_wedge_to_full_bz(E_iw, g_iw, pos[m.src])
    kr = m.reduced()
    for v in range(len(k)):
        s = m.src[v]
        assert np.array_equal(E[v], E_iw[pos[s]])
        ok, perm, sign = oracle.symmetry_operation(kr[s], kr[v])
        ref = np.array([[sign[j] * gg[perm[j]] for j in range(3)] for gg in g_iw[pos[s]]])
        assert np.array_equal(g[v], ref)


@pytest.mark.gpu
def test_band_structure_over_a_symmetric_mesh(gpu, oracle):
    """Si local, FP64: wedge solves distributed to the full zone equal direct solves at every vertex
    (energies 1e-10 eV; gradients 1e-8 of their scale for bands 5 meV from their neighbours), and the
    device gather equals the host one."""
    import torch

    si = _si()
    k = _star_set(6, 21)
    m = MeshBZ(si).set_vertices(k)
    bs = api.BandStructure()
    bs.Initialize(si, 8, k[:1], 9, False, False)
    E, g = m.compute_band_structure_over_mesh(bs, use_iwedge=True)
    assert len(m.iw_vertices) < len(k) / 10
    direct = api.BandStructure()
    direct.Initialize(si, 9, m.reduced(), 9, False, False)  # one band more, for the gap above band 8
    direct.Compute_parallel(True)
    direct.AdjustValues(False)
    Ed9, gd9 = np.asarray(direct.get_band_energies()), np.asarray(direct.get_band_energy_gradients())
    Ed, gd = Ed9[:, :8], gd9[:, :8]
    # AdjustValues shifts by the same VBM (a wedge point carries it) up to the solve's rounding
    assert np.abs(E - Ed).max() <= 1e-10
    # bands at least 5 meV from both neighbours (their gradients do not depend on a vector choice)
    gaps = np.minimum(np.diff(Ed9, axis=1, prepend=-1e9)[:, :8], np.diff(Ed9, axis=1)[:, :8])
    ok = gaps > 5e-3
    assert np.abs(g - gd)[ok].max() <= 1e-8 * np.abs(gd).max()
    # device gather
    used = np.asarray(m.iw_vertices)
    pos = np.full(len(k), -1)
    pos[used] = np.arange(len(used))
    Eiw = torch.from_numpy(np.ascontiguousarray(E[used])).cuda()
    giw = torch.from_numpy(np.ascontiguousarray(g[used])).cuda()
    dE, dg = m.distribute_on_device(Eiw, giw, pos[m.src])
    torch.cuda.synchronize()
    assert np.array_equal(dE.cpu().numpy(), E) and np.array_equal(dg.cpu().numpy(), g)


def _small_mesh(tmp_path, seed=3):
    """A mesh file (ASCII MSH 4.1, 8 nodes, 5 tetrahedra of a cube) read into a MeshBZ, with
    synthetic band energies (4 valence bands <= 0.1 eV at the first vertex, 3 conduction) and
    gradients on its vertices."""
    cube = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float) * 0.3
    tets = np.array([[1, 2, 4, 5], [2, 3, 4, 7], [2, 5, 6, 7], [4, 5, 7, 8], [2, 4, 5, 7]])
    src = tmp_path / "cube.msh"
    with open(src, "w") as f:
        f.write("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n$Nodes\n1 8 1 8\n3 1 0 8\n")
        f.write("".join(f"{i}\n" for i in range(1, 9)))
        f.write("".join(f"{x} {y} {z}\n" for x, y, z in cube))
        f.write("$EndNodes\n$Elements\n1 5 1 5\n3 1 4 5\n")
        f.write("".join(f"{e + 1} " + " ".join(str(v) for v in t) + "\n" for e, t in enumerate(tets)))
        f.write("$EndElements\n")
    m = MeshBZ(_si()).read_mesh_geometry_from_msh_file(str(src))
    rng = np.random.default_rng(seed)
    E = np.concatenate([np.sort(rng.uniform(-12.0, 0.0, (8, 4)), axis=1), 1.0 + np.sort(rng.uniform(0.0, 5.0, (8, 3)), axis=1)],
                       axis=1)
    E[0, 3] = 0.0  # the valence maximum at the first vertex, as after AdjustValues
    m.energies, m.gradients = E, rng.standard_normal((8, 7, 3)) * 1e-29
    return m, src


def test_gmsh_band_views_follow_the_reference_order(tmp_path):
    """MeshBZ::export_selected_bands_to_gmsh (bz_mesh.cpp:1426-1549): the mesh once, then band_<i>
    views, valence from the highest down (or from the lowest up), then conduction; gradients as
    3-component views after their band; values read back exactly; a second export appends views
    without rewriting the mesh."""
    from ultimateepm_gb300.mesh import read_msh_node_data, read_msh_tetrahedra

    m, src = _small_mesh(tmp_path)
    assert m.band_ranges() == ((0, 4), (4, 3))
    out = tmp_path / "bands.msh"
    order = m.export_selected_bands_to_gmsh(str(out), 2, 2, highest_valence_as_band0=True, write_gradients=True)
    assert order == [3, 2, 4, 5]
    tags, xyz = read_msh_nodes(str(out))
    t0, x0 = read_msh_nodes(str(src))
    assert (tags == t0).all() and np.array_equal(xyz, x0)
    assert np.array_equal(read_msh_tetrahedra(str(out)), read_msh_tetrahedra(str(src)))
    views = read_msh_node_data(str(out))
    assert [(v[0], v[1]) for v in views] == [("band_0", 1), ("grad_band_0", 3), ("band_1", 1), ("grad_band_1", 3),
                                             ("band_2", 1), ("grad_band_2", 3), ("band_3", 1), ("grad_band_3", 3)]
    for q, g in enumerate(order):
        assert np.array_equal(views[2 * q][3][:, 0], m.energies[:, g])
        assert np.array_equal(views[2 * q + 1][3], m.gradients[:, g, :])
    order2 = m.export_selected_bands_to_gmsh(str(out), 3, 0, highest_valence_as_band0=False)
    assert order2 == [0, 1, 2]
    text = open(out).read()
    assert text.count("$Nodes") == 1 and text.count("$NodeData") == 11
    # read back as the reference's loader does: bands in file order, valence by the first value
    back = MeshBZ(_si()).read_mesh_geometry_from_msh_file(str(out))
    Eb, gb = back.read_mesh_bands_from_msh_file(str(out))
    assert Eb.shape == (8, 7) and gb is None  # 7 bands, 4 gradient views
    assert np.array_equal(Eb[:, :4], m.energies[:, order])
    with pytest.raises(IndexError):
        m.export_selected_bands_to_gmsh(str(tmp_path / "x.msh"), 0, 4)
