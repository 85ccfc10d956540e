"""The committed steady states (tests/golden/make_steady.py) are steady
states of the oracle: the oracle's residual on them sits at its round-off
floor, and their stored Cf and J are the oracle's own on that state.  CPU."""
import json
import os

import numpy as np
import pytest

from structured_gb300 import case as C

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name,floor", [("steady_laminar_129x65", 1e-10), ("steady_sa_69x49", 5e-7)])
def test_steady_fixture_is_the_oracles_steady_state(port_built, name, floor):
    from oracle.port import PortCase
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    c = C.case_from_dict(json.loads(str(d["case"])))
    port = PortCase(c, d["xv"], d["yv"])
    r = port.residual(d["q"])
    norms = np.sqrt((r ** 2).sum(axis=(0, 1)))
    assert norms.max() < floor
    assert norms.max() < 1e-12 * d["hist"][0]
    cf, J = port.skin_friction(d["q"])
    assert np.array_equal(cf, d["cf"]) and J == float(d["J"])
