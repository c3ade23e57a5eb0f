"""The reference's material test cases (tests/test_material.cpp) on the product's Material
(turbomodal_gb300.meshgen.Material): validation (src/material.cpp:15-22, std::invalid_argument ->
ValueError) and the linear E(T) of at_temperature (src/material.cpp:33-38)."""

import pytest

from turbomodal_gb300.meshgen import Material


@pytest.mark.parametrize("E,nu,rho", [(-1e9, 0.3, 7800.0), (0.0, 0.3, 7800.0), (200e9, 0.0, 7800.0),
                                      (200e9, -0.1, 7800.0), (200e9, 0.5, 7800.0), (200e9, 0.6, 7800.0),
                                      (200e9, 0.3, -1.0), (200e9, 0.3, 0.0)])
def test_rejects_invalid(E, nu, rho):
    with pytest.raises(ValueError):
        Material(E, nu, rho)


def test_construction_and_temperature():
    m = Material(200e9, 0.3, 7800.0, 293.15, -5e7)
    assert (m.E, m.nu, m.rho, m.T_ref, m.E_slope) == (200e9, 0.3, 7800.0, 293.15, -5e7)
    assert m.at_temperature(293.15).E == 200e9
    hot = m.at_temperature(793.15)
    assert hot.E == pytest.approx(200e9 - 5e7 * 500) and hot.nu == 0.3 and hot.rho == 7800.0
    assert Material(200e9, 0.3, 7800.0, 293.15, 5e7).at_temperature(393.15).E > 200e9
    assert Material(200e9, 0.3, 7800.0).at_temperature(1000.0).E == 200e9
    with pytest.raises(RuntimeError):
        m.at_temperature(293.15 + 5000.0)
