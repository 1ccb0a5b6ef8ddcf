"""Band structure over a Brillouin-zone mesh: the caller behind the reference's BandsOnBZ.

Mirrors MeshBZ (src/BZ_MESH/bz_mesh.cpp) for the band-structure part:
  read_mesh_geometry_from_msh_file   the mesh vertices, scaled by 2 pi / a when asked (:67-105);
                                     read here from the MSH file itself (ASCII 4.1 or 2.2 $Nodes),
                                     in the node order gmsh returns them
  is_irreducible_wedge               z >= 0, z <= y <= x <= 1, x + y + z <= 3/2 in reduced units (:1176)
  load_kstar_ibz_to_bz               the reference's "<mesh>_kstar_ibz_to_bz.txt" (:198-271)
  build_kstar_ibz_to_bz              the same map computed here: every vertex folded into the wedge
                                     (absolute values, sorted descending) and matched to a wedge vertex
  compute_band_structure_over_mesh   solve the wedge (or every) vertex, AdjustValues, then the wedge
                                     -> full-zone distribution (:1230-1303)
  distribute_energies_from_iw_wedge_to_full_bz
                                     energies copied, gradients taken through the signed permutation
                                     apply_same_symmetry_operation finds (:1312-1414): on the host, or
                                     as one device gather (uepm_star_expand_device) after a device solve
  export_selected_bands_to_gmsh      the band views (:1426-1549): the mesh once, then one node-data
                                     view per exported band ("band_<i>"), and per gradient
                                     ("grad_band_<i>", 3 components), valence bands first (highest as
                                     band 0 on request), then conduction bands; written as ASCII MSH
                                     4.1 (the reference lets gmsh write binary; gmsh reads both)
  read_mesh_bands_from_msh_file      the views back, classified as the reference does (:330-392): a
                                     band is valence when its value at the first vertex is <= 0.1 eV
Energies in eV, gradients in eV m (the reference's units), vertex positions in SI (1/m).
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import _native as N


def read_msh_nodes(path: str) -> tuple[np.ndarray, np.ndarray]:
    """Node tags and coordinates (n x 3) of an ASCII MSH 4.1 or 2.2 file, in file order."""
    with open(path, "r") as f:
        lines = f.read().splitlines()
    ver = None
    i = 0
    while i < len(lines):
        t = lines[i].strip()
        if t == "$MeshFormat":
            parts = lines[i + 1].split()
            ver, ftype = float(parts[0]), int(parts[1])
            if ftype != 0:
                raise ValueError("binary MSH files are not supported; save the mesh as ASCII")
            i += 2
            continue
        if t == "$Nodes":
            if ver is None:
                raise ValueError("$Nodes before $MeshFormat")
            i += 1
            if ver >= 4.0:
                nblocks, nnodes = (int(x) for x in lines[i].split()[:2])
                i += 1
                tags = np.empty(nnodes, dtype=np.int64)
                xyz = np.empty((nnodes, 3))
                pos = 0
                for _ in range(nblocks):
                    _, _, param, nin = (int(x) for x in lines[i].split()[:4])
                    i += 1
                    tags[pos:pos + nin] = [int(lines[i + q]) for q in range(nin)]
                    i += nin
                    for q in range(nin):
                        xyz[pos + q] = [float(x) for x in lines[i + q].split()[:3]]
                    i += nin
                    pos += nin
                    del param
                return tags, xyz
            n = int(lines[i])
            i += 1
            tags = np.empty(n, dtype=np.int64)
            xyz = np.empty((n, 3))
            for q in range(n):
                p = lines[i + q].split()
                tags[q] = int(p[0])
                xyz[q] = [float(x) for x in p[1:4]]
            return tags, xyz
        i += 1
    raise ValueError(f"{path}: no $Nodes section")


def read_msh_tetrahedra(path: str) -> np.ndarray:
    """Node tags (n x 4) of the 4-node tetrahedra (element type 4) of an ASCII MSH 4.1 or 2.2 file, in
    file order: the elements gmsh::model::mesh::getElements(dim = 3) returns to MeshBZ
    (bz_mesh.cpp:106-120)."""
    with open(path, "r") as f:
        lines = f.read().splitlines()
    ver = None
    i = 0
    while i < len(lines):
        t = lines[i].strip()
        if t == "$MeshFormat":
            parts = lines[i + 1].split()
            ver, ftype = float(parts[0]), int(parts[1])
            if ftype != 0:
                raise ValueError("binary MSH files are not supported; save the mesh as ASCII")
            i += 2
            continue
        if t == "$Elements":
            if ver is None:
                raise ValueError("$Elements before $MeshFormat")
            i += 1
            out = []
            if ver >= 4.0:
                nblocks = int(lines[i].split()[0])
                i += 1
                for _ in range(nblocks):
                    dim, _, etype, nin = (int(x) for x in lines[i].split()[:4])
                    i += 1
                    if dim == 3 and etype == 4:
                        out.extend([int(x) for x in lines[i + q].split()[1:5]] for q in range(nin))
                    i += nin
            else:
                n = int(lines[i])
                i += 1
                for q in range(n):
                    p = [int(x) for x in lines[i + q].split()]
                    if p[1] == 4:
                        out.append(p[3 + p[2]:3 + p[2] + 4])
            return np.array(out, dtype=np.int64).reshape(-1, 4)
        i += 1
    raise ValueError(f"{path}: no $Elements section")


def read_msh_node_data(path: str) -> list[tuple[str, int, np.ndarray, np.ndarray]]:
    """The $NodeData views of an ASCII MSH file in file order: (name, components, node tags, values
    [n][components])."""
    with open(path, "r") as f:
        lines = f.read().splitlines()
    out = []
    i = 0
    while i < len(lines):
        if lines[i].strip() != "$NodeData":
            i += 1
            continue
        i += 1
        ns = int(lines[i]); i += 1
        strs = [lines[i + q].strip().strip('"') for q in range(ns)]; i += ns
        nr = int(lines[i]); i += 1 + nr
        ni = int(lines[i]); i += 1
        ints = [int(lines[i + q]) for q in range(ni)]; i += ni
        ncomp, nn = ints[1], ints[2]
        tags = np.empty(nn, dtype=np.int64)
        vals = np.empty((nn, ncomp))
        for q in range(nn):
            p = lines[i + q].split()
            tags[q] = int(p[0])
            vals[q] = [float(x) for x in p[1:1 + ncomp]]
        i += nn
        if lines[i].strip() != "$EndNodeData":
            raise ValueError(f"{path}: malformed $NodeData")
        out.append((strs[0] if strs else "", ncomp, tags, vals))
        i += 1
    return out


def tetra_signed_volumes(positions: np.ndarray, tetra: np.ndarray) -> np.ndarray:
    """Tetra::compute_signed_volume (mesh_tetra.cpp:128-132): (1/6) e0 . (e1 x e2) with
    e_j = v_{j+1} - v_0."""
    p = positions[tetra]
    e0, e1, e2 = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]
    c = np.stack([e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1], e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                  e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], axis=1)
    return (1.0 / 6.0) * np.einsum("ij,ij->i", e0, c)


def _fold_key(kr: np.ndarray, digits: int) -> list[tuple]:
    f = -np.sort(-np.abs(kr), axis=1)  # |k| sorted descending: the wedge representative
    return [tuple(r) for r in np.round(f, digits)]


class MeshBZ:
    def __init__(self, material):
        """material: api.Material (its lattice constant sets the SI <-> reduced scale)."""
        self.material = material
        self.positions = np.zeros((0, 3))  # SI
        self.node_tags = np.zeros(0, dtype=np.int64)
        self.kstar: list[list[int]] = []  # indexed by wedge vertex
        self.iw_vertices: list[int] = []
        self.energies = None
        self.gradients = None
        self.tetra = np.zeros((0, 4), dtype=np.int64)
        self.tetra_volumes = np.zeros(0)

    # ---- geometry --------------------------------------------------------------------------------
    def si_to_reduced_scale(self) -> float:
        return self.material.get_lattice_constant_meter() / (2.0 * math.pi)

    def read_mesh_geometry_from_msh_file(self, filename: str, normalize_by_fourier_factor: bool = True):
        tags, xyz = read_msh_nodes(filename)
        f = 2.0 * math.pi / self.material.get_lattice_constant_meter() if normalize_by_fourier_factor else 1.0
        self.node_tags = tags
        self.positions = xyz * f
        self.filename = filename
        self._file_xyz = xyz  # the model's own coordinates, for writing the mesh back
        try:
            raw = read_msh_tetrahedra(filename)
            self._file_tetra = raw
            self.set_tetrahedra(raw - 1)  # vertex = node tag - 1 (bz_mesh.cpp:135-138)
        except ValueError:
            self._file_tetra = np.zeros((0, 4), dtype=np.int64)
            self.tetra = np.zeros((0, 4), dtype=np.int64)
            self.tetra_volumes = np.zeros(0)
        return self

    def set_tetrahedra(self, vertex_indices: np.ndarray):
        """Tetrahedra as vertex indices (m x 4); those with |signed volume| < 1e-12 are dropped, as
        MeshBZ does when it reads them (bz_mesh.cpp:130-146)."""
        t = np.asarray(vertex_indices, dtype=np.int64).reshape(-1, 4)
        if len(t) and (t.min() < 0 or t.max() >= len(self.positions)):
            raise ValueError("tetrahedron vertex index out of range")
        vol = tetra_signed_volumes(self.positions, t) if len(t) else np.zeros(0)
        keep = np.abs(vol) >= 1e-12
        self.tetra = t[keep]
        self.tetra_volumes = vol[keep]
        return self

    def set_vertices(self, k_reduced: np.ndarray):
        """Vertices given directly as reduced k-points (n x 3)."""
        self.positions = np.asarray(k_reduced, dtype=np.float64) / self.si_to_reduced_scale()
        self.node_tags = np.arange(1, len(self.positions) + 1)
        return self

    def reduced(self) -> np.ndarray:
        return self.positions * self.si_to_reduced_scale()

    def is_irreducible_wedge(self, k_si: np.ndarray) -> np.ndarray:
        k = np.atleast_2d(np.asarray(k_si, dtype=np.float64)) * self.si_to_reduced_scale()
        x, y, z = k[:, 0], k[:, 1], k[:, 2]
        eps = 1e-12
        return (z >= -eps) & (z <= y + eps) & (y <= x + eps) & (x <= 1.0 + eps) & ((x + y + z) <= 1.5 + eps)

    # ---- band views (gmsh node data) --------------------------------------------------------------
    def band_ranges(self) -> tuple[tuple[int, int], tuple[int, int]]:
        """(first index, count) of the valence and of the conduction bands, by the reference's rule
        (bz_mesh.cpp:365-378): band b is valence when its energy at the first vertex is <= 0.1 eV."""
        if self.energies is None:
            raise RuntimeError("no band energies on the mesh")
        E = np.asarray(self.energies)
        val = [b for b in range(E.shape[1]) if E[0, b] <= 0.1]
        con = [b for b in range(E.shape[1]) if E[0, b] > 0.1]
        return (val[0] if val else -1, len(val)), (con[0] if con else -1, len(con))

    def _write_mesh_msh41(self, f):
        tags = np.asarray(self.node_tags, dtype=np.int64)
        xyz = getattr(self, "_file_xyz", None)
        if xyz is None:
            xyz = self.positions
        tet = getattr(self, "_file_tetra", None)
        if tet is None:
            tet = self.tetra + 1
        f.write("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n")
        f.write(f"$Nodes\n1 {len(tags)} {int(tags.min())} {int(tags.max())}\n3 1 0 {len(tags)}\n")
        f.write("".join(f"{int(t)}\n" for t in tags))
        f.write("".join(f"{x!r} {y!r} {z!r}\n" for x, y, z in np.asarray(xyz, dtype=np.float64).tolist()))
        f.write("$EndNodes\n")
        f.write(f"$Elements\n1 {len(tet)} 1 {len(tet)}\n3 1 4 {len(tet)}\n")
        f.write("".join(f"{e + 1} {a} {b} {c} {d}\n" for e, (a, b, c, d) in enumerate(np.asarray(tet).tolist())))
        f.write("$EndElements\n")

    def _write_view(self, f, name: str, vals: np.ndarray):
        vals = np.asarray(vals, dtype=np.float64).reshape(len(self.node_tags), -1)
        f.write(f'$NodeData\n1\n"{name}"\n1\n0\n3\n0\n{vals.shape[1]}\n{len(self.node_tags)}\n')
        f.write("".join(f"{int(t)} " + " ".join(repr(x) for x in row) + "\n"
                        for t, row in zip(np.asarray(self.node_tags).tolist(), vals.tolist())))
        f.write("$EndNodeData\n")

    def export_selected_bands_to_gmsh(self, out_filename: str, nb_valence_to_export: int, nb_conduction_to_export: int,
                                      highest_valence_as_band0: bool = True, model_name_or_msh_path: str = "",
                                      write_gradients: bool = False):
        """MeshBZ::export_selected_bands_to_gmsh (bz_mesh.cpp:1426-1549). The mesh is written only when
        out_filename does not exist yet; the views are appended. Valence bands: from the highest down
        when highest_valence_as_band0, else from the lowest up; then the conduction bands in order.
        Views are named band_<i> (and grad_band_<i>) with i counting the exported bands. Values are
        written with 17 significant digits (they read back exactly). model_name_or_msh_path is
        accepted for signature compatibility: the mesh written is the one this object read."""
        del model_name_or_msh_path
        if len(self.node_tags) == 0 or self.energies is None or len(self.energies) != len(self.node_tags):
            raise RuntimeError("Mesh vertices/tags not initialized or inconsistent.")
        E = np.asarray(self.energies)
        G = None if self.gradients is None else np.asarray(self.gradients)
        if write_gradients and G is None:
            raise RuntimeError("Vertex gradient vector too small for requested band index.")
        (v0, nv), (c0, nc) = self.band_ranges()
        order = []
        if nb_valence_to_export > 0:
            if highest_valence_as_band0:
                last = v0 + nv - 1
                order += list(range(last, last - int(nb_valence_to_export), -1))
            else:
                order += list(range(v0, v0 + int(nb_valence_to_export)))
        for g in range(int(nb_conduction_to_export)):
            if g >= nc:
                raise IndexError("conduction band index out of range")  # get_global_band_index throws
            order.append(c0 + g)
        for g in order:
            if g < 0 or g >= E.shape[1]:
                raise RuntimeError("Vertex band vector too small for requested band index.")
        write_mesh = not os.path.exists(out_filename)
        with open(out_filename, "a") as f:
            if write_mesh:
                self._write_mesh_msh41(f)
            for idx, g in enumerate(order):
                self._write_view(f, f"band_{idx}", E[:, g])
                if write_gradients:
                    self._write_view(f, f"grad_band_{idx}", G[:, g, :])
        return order

    def read_mesh_bands_from_msh_file(self, filename: str):
        """MeshBZ::read_mesh_bands_from_msh_file (bz_mesh.cpp:330-392): every 1-component view is a band
        (valence when its first value is <= 0.1 eV), every 3-component view the gradient of the band
        before it. Returns (energies [n][nb], gradients [n][nb][3] or None) and keeps them."""
        bands, grads = [], []
        for name, ncomp, tags, vals in read_msh_node_data(filename):
            if ncomp == 1:
                bands.append(vals[:, 0])
            elif ncomp == 3:
                grads.append(vals)
            else:
                raise RuntimeError(f"read_mesh_bands_from_msh_file: unsupported number of components per view: {ncomp}")
        self.energies = np.stack(bands, axis=1) if bands else None
        self.gradients = np.stack(grads, axis=1) if grads and len(grads) == len(bands) else None
        return self.energies, self.gradients

    # ---- the k-star of every wedge vertex ---------------------------------------------------------
    def build_kstar_ibz_to_bz(self, digits: int = 9):
        """Maps each wedge vertex to the vertices of its star: every vertex folded into the wedge is
        matched to the wedge vertex at the same reduced position (rounded to `digits` places)."""
        kr = self.reduced()
        inw = np.nonzero(self.is_irreducible_wedge(self.positions))[0]
        if len(inw) == 0:
            raise RuntimeError("No vertices in irreducible wedge. Cannot distribute energies to full BZ.")
        where = {}
        for idx, key in zip(inw, _fold_key(kr[inw], digits)):
            where.setdefault(key, int(idx))
        src = np.empty(len(kr), dtype=np.int64)
        for v, key in enumerate(_fold_key(kr, digits)):
            if key not in where:
                raise RuntimeError(f"vertex {v} at {kr[v]} has no image in the irreducible wedge: the mesh is not "
                                   "symmetric under the cubic group")
            src[v] = where[key]
        self._set_star(src)
        return self

    def load_kstar_ibz_to_bz(self, filename: str):
        """The reference's kstar file: lines "iw m id_1 ... id_m" (comments '#')."""
        rows = []
        with open(filename) as f:
            for line in f:
                if not line.strip() or line.startswith("#"):
                    continue
                p = line.split()
                iw, m = int(p[0]), int(p[1])
                rows.append((iw, [int(x) for x in p[2:2 + m]]))
        n = len(self.positions)
        src = np.full(n, -1, dtype=np.int64)
        inw = self.is_irreducible_wedge(self.positions)
        for iw, ids in rows:
            if not inw[iw]:
                raise RuntimeError(f"load_kstar_file: vertex {iw} does not lie in the irreducible wedge, but it should")
            for v in ids:
                if v >= n:
                    raise RuntimeError(f"load_kstar_file: index {v} out of range")
                src[v] = iw
        if (src < 0).any():
            raise RuntimeError("load_kstar_file: number of k-points in IBZ does not match number of vertices in mesh")
        self._set_star(src)
        return self

    def _set_star(self, src: np.ndarray):
        self.src = src
        self.iw_vertices = sorted(set(int(s) for s in src))
        self.kstar = {iw: [] for iw in self.iw_vertices}
        for v, s in enumerate(src):
            self.kstar[int(s)].append(v)
        # signed permutation of every vertex relative to its wedge source (host C ABI)
        L = N.load()
        kr = np.ascontiguousarray(self.reduced())
        ks = np.ascontiguousarray(kr[src])
        self.ops = np.zeros(len(kr), dtype=np.uint16)
        found = np.zeros(len(kr), dtype=np.int32)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        N.check(L.uepm_star_operations(dp(ks), dp(kr), len(kr), self.ops.ctypes.data_as(C.POINTER(C.c_uint16)),
                                       found.ctypes.data_as(C.POINTER(C.c_int32))))
        self.ops_found = found.astype(bool)

    # ---- band structure ----------------------------------------------------------------------------
    def compute_band_structure_over_mesh(self, band_structure, use_iwedge: bool = True):
        """band_structure: an api.BandStructure already Initialize-d (material, bands, basis, flags).
        Solves the wedge vertices (or all of them), with gradients, shifts by AdjustValues(False), and
        distributes to the full zone. Returns (energies [n][nb], gradients [n][nb][3])."""
        kr = self.reduced()
        if use_iwedge:
            if not self.iw_vertices:
                self.build_kstar_ibz_to_bz()
            used = np.asarray(self.iw_vertices, dtype=np.int64)
        else:
            used = np.arange(len(kr))
        band_structure.set_kpoints(np.ascontiguousarray(kr[used]))
        band_structure.Compute_parallel(True)
        band_structure.AdjustValues(False)
        E = np.asarray(band_structure.get_band_energies())
        g = np.asarray(band_structure.get_band_energy_gradients())
        if not use_iwedge:
            self.energies, self.gradients = E, g
            return E, g
        pos = np.full(len(kr), -1, dtype=np.int64)
        pos[used] = np.arange(len(used))
        self.energies, self.gradients = self.distribute_energies_from_iw_wedge_to_full_bz(E, g, pos[self.src])
        return self.energies, self.gradients

    def distribute_energies_from_iw_wedge_to_full_bz(self, E_iw: np.ndarray, g_iw: np.ndarray, src_rows: np.ndarray):
        """Host gather: rows src_rows[v] of the wedge results for every vertex v, gradients through
        the vertex's signed permutation."""
        E = E_iw[src_rows]
        perm = np.stack([(self.ops >> (2 * j)) & 3 for j in range(3)], axis=1).astype(np.int64)
        sign = np.stack([np.where((self.ops >> (6 + j)) & 1, -1.0, 1.0) for j in range(3)], axis=1)
        gs = g_iw[src_rows]  # [n][nb][3]
        g = np.take_along_axis(gs, perm[:, None, :].repeat(gs.shape[1], axis=1), axis=2) * sign[:, None, :]
        return E, g

    def distribute_on_device(self, dE_iw, dg_iw, src_rows, stream=None):
        """Device gather with uepm_star_expand_device: dE_iw [m][nb], dg_iw [m][nb][3] (torch CUDA
        tensors, float64), src_rows [n] wedge rows. Returns device tensors (E [n][nb], g [n][nb][3])."""
        import torch

        L = N.load()
        n, nb = len(src_rows), dE_iw.shape[1]
        dev = dE_iw.device
        d_src = torch.from_numpy(np.ascontiguousarray(src_rows, dtype=np.int64)).to(dev)
        d_op = torch.from_numpy(self.ops.astype(np.int16)).to(dev)
        E = torch.empty((n, nb), dtype=torch.float64, device=dev)
        g = torch.empty((n, nb, 3), dtype=torch.float64, device=dev) if dg_iw is not None else None
        s = stream if stream is not None else torch.cuda.current_stream()
        p = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
        N.check(L.uepm_star_expand_device(p(dE_iw), p(dg_iw), p(d_src), p(d_op), n, nb, p(E), p(g),
                                          C.c_void_p(s.cuda_stream)))
        return E, g
