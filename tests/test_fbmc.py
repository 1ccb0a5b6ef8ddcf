"""On-demand band queries for FBMC particles (src/FBMC/particle.cpp:52-63): energy and group
velocity v = grad E / h_bar_eV at each particle's k (SI) and band, against the oracle."""
import os

import numpy as np
import pytest

from ultimateepm_gb300 import _native as N
from ultimateepm_gb300 import api
from ultimateepm_gb300.fbmc import H_BAR_EV, BandQuery


def test_h_bar_ev_is_the_reference_constant(oracle):
    # h_bar / eV_to_J (src/Common/physical_constants.hpp:26-28)
    assert H_BAR_EV == oracle.H_BAR / oracle.Q_E


@pytest.mark.gpu
@pytest.mark.parametrize("device", [False, True])
def test_energy_and_velocity_match_the_oracle(gpu, oracle, mats, device):
    si = api.Material("Si", raw=N.UepmMaterial.from_buffer_copy(bytes(mats["Si-CB"])))
    G = oracle.generate_basis(10)
    bq = BandQuery(si, basis=G)
    a = si.get_lattice_constant_meter()
    kr = oracle.sample_first_bz(64, 21)
    bands = np.random.default_rng(2).integers(0, 12, len(kr))
    k_si = kr * (2 * np.pi / a)
    if device:
        import torch

        E, v = bq.energy_and_velocity_device(torch.from_numpy(k_si).cuda(), torch.from_numpy(bands).cuda())
        E, v = E.cpu().numpy(), v.cpu().numpy()
    else:
        E, v = bq.energy_and_velocity(k_si, bands)
    ref = oracle.band_structure(mats["Si-CB"], G, kr, 12, grad=True)
    rows = np.arange(len(kr))
    np.testing.assert_allclose(E, ref["E"][rows, bands], rtol=0, atol=1e-10)
    vref = ref["grad"][rows, bands] / H_BAR_EV
    scale = np.abs(vref).max()
    np.testing.assert_allclose(v, vref, rtol=0, atol=1e-8 * scale)
    with pytest.raises(IndexError):
        bq.energy_and_velocity(k_si[:1], [G.shape[0]])
    with pytest.raises(ValueError):
        bq.energy_and_velocity(k_si[:2], [0])
    bq.close()
