"""Host-side pieces of the product checked against the oracle and the reference's own code
(golden fixtures), plus the C ABI symbol table. CPU only: no compute call touches a GPU."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, PARAMS, ROOT


def test_abi_exports_every_declared_symbol(native):
    header = open(os.path.join(ROOT, "include", "uepm_gb300.h")).read()
    declared = set(re.findall(r"\b(uepm_[a-z_]+)\s*\(", header))
    assert declared, "no declarations parsed"
    for name in sorted(declared):
        assert hasattr(native, name), f"{name} declared in uepm_gb300.h but not exported"
    from ultimateepm_gb300 import _native

    assert declared == set(_native.EXPORTED)


def test_material_layout(native):
    from ultimateepm_gb300 import _native

    assert native.uepm_material_size() == C.sizeof(_native.UepmMaterial)


@pytest.mark.parametrize("shells", [2, 3, 8, 9, 10, 11, 12, 13, 20, 116])
def test_basis_matches_oracle(native, oracle, shells):
    from ultimateepm_gb300 import generate_basis_vectors

    np.testing.assert_array_equal(generate_basis_vectors(shells), oracle.generate_basis(shells))


def test_basis_rejects_out_of_range(native):
    from ultimateepm_gb300 import generate_basis_vectors

    for bad in (0, 1, 117):
        with pytest.raises(RuntimeError):
            generate_basis_vectors(bad)


def test_path_matches_reference_code(native):
    from ultimateepm_gb300 import SymmetryPoints

    for e in json.load(open(os.path.join(GOLDEN, "ref_paths.json"))):
        if e["count"] < 0:
            with pytest.raises(ValueError):
                SymmetryPoints().GeneratePoints(list(e["labels"]), e["n"])
            continue
        k, pos = SymmetryPoints().GeneratePoints(list(e["labels"]), e["n"])
        np.testing.assert_array_equal(k.ravel(), np.array(e["k"]))
        assert pos == e["sym"]


@pytest.mark.parametrize("fname", ["materials.yaml", "si-cohen-bergstresser.yaml", "si-nonlocal-d.yaml"])
def test_yaml_loader_matches_oracle_reader(native, oracle, fname):
    from ultimateepm_gb300 import Materials

    m = Materials()
    m.load_material_parameters(os.path.join(PARAMS, fname))
    ref = oracle.load_materials(os.path.join(PARAMS, fname))
    assert list(m.materials) == list(ref)
    for sym in ref:
        assert bytes(m.materials[sym].raw) == bytes(ref[sym]), sym


def test_yaml_loader_errors(native, tmp_path):
    from ultimateepm_gb300 import Materials

    with pytest.raises(ValueError):
        Materials().load_material_parameters(str(tmp_path / "missing.yaml"))
    bad = tmp_path / "bad.yaml"
    bad.write_text("materials:\n  - name: X\n    symbol: X\n    lattice-constant: 5.0\n"
                   "    pseudo-potential-parameters:\n      V3S: -0.2\n")
    with pytest.raises(RuntimeError):
        Materials().load_material_parameters(str(bad))
    well = tmp_path / "well.yaml"
    well.write_text(open(os.path.join(PARAMS, "si-nonlocal-d.yaml")).read().replace('"square"', '"round"'))
    with pytest.raises(RuntimeError):
        Materials().load_material_parameters(str(well))


@pytest.mark.parametrize("nb,soc,mcz", [(16, 0, 0), (16, 0, 1), (12, 1, 0), (4, 0, 0), (3, 0, 0), (2, 0, 1), (1, 0, 0)])
def test_adjust_values_matches_oracle(native, oracle, nb, soc, mcz):
    from ultimateepm_gb300 import _native

    rng = np.random.default_rng(nb * 7 + soc)
    E = np.sort(rng.normal(size=(50, nb)) * 3 + np.arange(nb) * 1.5, axis=1)
    E1 = E.copy()
    E2 = E.copy()
    gap_o, found_o = oracle.adjust_values(E1, soc=bool(soc), min_cond_zero=bool(mcz))
    gap = C.c_double()
    found = C.c_int32()
    native.uepm_adjust_values(E2.ctypes.data_as(C.POINTER(C.c_double)), E2.shape[0], nb, soc, mcz, C.byref(gap),
                              C.byref(found))
    assert bool(found.value) == found_o
    assert gap.value == gap_o
    np.testing.assert_array_equal(E2, E1)


def test_no_cpu_fallback_when_library_missing(monkeypatch, tmp_path):
    """The binding refuses to run without the native library (it never computes on the CPU)."""
    import ultimateepm_gb300._native as nat

    monkeypatch.setattr(nat, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(nat, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        nat.load()
    # monkeypatch restores the path and the loaded library afterwards


def test_product_loader_equals_the_reference_loader(native):
    """uepm_materials_load against Materials::load_material_parameters of the reference itself
    (Material.cpp:33-71 compiled against oracle/shim; fixture tests/golden/ref_materials.json)."""
    from ultimateepm_gb300 import Materials

    ref = json.load(open(os.path.join(GOLDEN, "ref_materials.json")))
    for fname, mats in ref.items():
        m = Materials()
        m.load_material_parameters(os.path.join(PARAMS, fname))
        assert set(m.materials) == set(mats), fname
        for sym, fields in mats.items():
            for f, v in fields.items():
                assert getattr(m.materials[sym].raw, f) == v, (fname, sym, f)


@pytest.mark.parametrize("key,fname,sym,nb,labels,npts,shells,nl,soc", [
    ("si_local", "si-cohen-bergstresser.yaml", "Si", 16, "LGXWKULWXKG", 40, 10, 0, 0),
    ("ge_nl_soc", "materials.yaml", "Ge", 8, "LGX", 20, 8, 1, 1)])
def test_band_file_byte_identical_to_the_reference(native, tmp_path, key, fname, sym, nb, labels, npts, shells, nl,
                                                   soc):
    """BandStructure::export_result_in_file (BandStructure.cpp:290-314): the Python mirror's band file
    for the reference's own energies is byte-identical to the file the reference wrote."""
    from ultimateepm_gb300 import BandStructure, Materials

    mats = Materials()
    mats.load_material_parameters(os.path.join(PARAMS, fname))
    bs = BandStructure()
    bs.Initialize(mats.materials[sym], nb, list(labels), shells, bool(nl), bool(soc), nrPoints=npts)
    bs.m_energies = np.load(os.path.join(GOLDEN, "ref_bands.npz"))[key]
    out = tmp_path / "bands.txt"
    bs.export_result_in_file(str(out))
    assert out.read_bytes() == open(os.path.join(GOLDEN, f"ref_band_{key}.txt"), "rb").read()
