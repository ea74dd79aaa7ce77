"""Host-side mesh generator and seeded inputs against the oracle (CPU only)."""
import numpy as np
import pytest

import oracle as O
from gtgpu import mesh as M


@pytest.mark.parametrize("cells,simplex", [((3, 4), False), ((1, 1), False), ((2, 3, 4), False), ((1, 1, 1), False),
                                           ((3, 3, 3), True), ((4, 2, 3), True), ((64, 64), False)])
def test_cartesian_mesh_matches_oracle(cells, simplex):
    box = tuple(x for c in cells for x in (0.0, 1.5))
    a = M.cartesian_mesh(box, cells, simplexify=simplex)
    b = O.cartesian_mesh(box, cells, simplexify=simplex)
    assert np.array_equal(a.cell_nodes, b["cell_nodes"])
    assert np.array_equal(a.coords, b["coords"])
    assert np.array_equal(a.corners, b["pf0"])
    if len(cells) == 2:
        assert np.array_equal(a.bfaces, b["pf1"]) and np.array_equal(a.bface_group, b["pf1g"])
    else:
        assert np.array_equal(a.bfaces, b["pf2"]) and np.array_equal(a.bface_group, b["pf2g"])
        assert np.array_equal(a.bedges, b["pf1"])


def test_seeded_inputs_match_oracle():
    a = M.cartesian_mesh((0, 1, 0, 1, 0, 1), (5, 6, 7), simplexify=True)
    M.jitter_interior_nodes(a, 0.2, 202)
    b = O.cartesian_mesh((0, 1, 0, 1, 0, 1), (5, 6, 7), simplexify=True)
    O.jitter(b, 0.2, 202)
    assert np.array_equal(a.coords, b["coords"])
    k1, k2 = M.lognormal_cells(5000, 1.0, 202), O.lognormal_cells(5000, 1.0, 202)
    assert np.abs(k1 / k2 - 1).max() < 1e-14


def test_invalid_mesh_arguments():
    with pytest.raises(ValueError):
        M.cartesian_mesh((0, 1, 0, 1), (1, 3))
    with pytest.raises(NotImplementedError):
        M.cartesian_mesh((0, 1, 0, 1), (2, 2), simplexify=True)
