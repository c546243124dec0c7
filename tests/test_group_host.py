"""Host side of group contexts (several particles solved as one batch): argument checks made before any device work,
and the phase relation the GPU test relies on between a particle's incident field with its own box centre and with
the common box's centre as reference point (a constant factor of modulus 1)."""
import numpy as np
import pytest


def _setups(dpl2=10):
    import adda_gb300 as A
    return [A.Setup(grid=16, m=1.5, dpl=10), A.Setup(grid=12, shape="ellipsoid", pars=(0.8, 0.6), m=1.33 + 0.01j,
                                                    dpl=dpl2)]


def test_group_rejects_different_lattice_spacing():
    import adda_gb300 as A
    with pytest.raises(ValueError):
        A.Context.group(_setups(dpl2=12), rhs_per_particle=2)


def test_group_rejects_a_box_that_does_not_hold_every_particle():
    import adda_gb300 as A
    with pytest.raises(ValueError):
        A.Context.group(_setups(), rhs_per_particle=2, box=(16, 16, 8))


def test_common_box_plane_wave_is_a_constant_phase_of_the_own_box_one():
    import adda_gb300 as A
    setups = _setups()
    box = tuple(max(s.box[d] for s in setups) for d in range(3))
    for s in setups:
        for k, e in enumerate(s.incpol):
            eg = A.plane_wave(box, s.pos, s.gridspace, s.wavenum, s.prop, e)
            j = int(np.argmax(np.abs(s.einc[k])))
            ph = eg[j] / s.einc[k][j]
            assert abs(abs(ph) - 1) < 1e-12
            assert np.abs(eg - ph * s.einc[k]).max() < 1e-12
