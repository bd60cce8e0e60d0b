"""exnode/exelem export of a state (the reference's field export layout):
values and element topology read back exactly."""
import numpy as np
import pytest

from cm_gb300 import field_export as F
from cm_gb300 import mesh as M


@pytest.mark.parametrize("nxi,pmode", [(3, "node"), (2, "element")])
def test_export_round_trip(tmp_path, nxi, pmode):
    m = M.regular_box(2, 3, 2, nxi_u=nxi, pressure=pmode, perturb=0.1, seed=4)
    x = M.deformed_state(m, stretch=1.1, shear=0.05, noise=0.02, pressure=-1.3, seed=5)
    node_file, elem_file = F.export(str(tmp_path / "state"), m, x)
    vals = F.read_exnode_values(node_file)
    for n in range(m.nu):
        v = vals[0][n + 1]
        assert v[:3] == list(m.X[:, n])
        assert v[3:] == [x[c * m.nu + n] for c in range(3)]
    if pmode == "node":
        pnode = m.pressure_node_u()
        for q in range(m.np):
            assert vals[1][pnode[q] + 1] == [x[3 * m.nu + q]]
    elems = F.read_exelem_nodes(elem_file)
    assert len(elems) == m.ne
    for e in range(m.ne):
        assert elems[e + 1] == list(m.elem_u[e] + 1)
    text = open(elem_file).read()
    assert ("q.Lagrange*q.Lagrange*q.Lagrange" if nxi == 3 else "l.Lagrange*l.Lagrange*l.Lagrange") in text
    assert "coordinate, rectangular cartesian" in open(node_file).read()
