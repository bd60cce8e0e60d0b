"""exnode/exelem export of a state.

Both files are compared byte for byte with the reference's own writer,
src/FieldExport.c, compiled unchanged from the reference tree
(oracle/build.py build_ref) and driven the way the reference's
FIELD_IO_NODES_EXPORT / FIELD_IO_ELEMENTS_EXPORT drive it
(oracle/fieldexport_ref.py); those tests are skipped where the reference tree
is absent, and the files the reference writer produced for four small states,
committed under tests/golden/field_export with the script that wrote them,
are compared everywhere.  Values and element topology also read back exactly.
"""
import os

import numpy as np
import pytest

from cm_gb300 import field_export as F
from cm_gb300 import mesh as M


@pytest.mark.parametrize("nxi,pmode", [(3, "node"), (2, "element"), (2, "node")])
def test_exnode_matches_the_reference_writer(tmp_path, nxi, pmode):
    import build as ob  # oracle/build.py
    if ob.build_ref() is None:
        pytest.skip("the reference tree is not on this machine")
    import fieldexport_ref as R  # oracle/fieldexport_ref.py
    m = M.regular_box(2, 3, 2, nxi_u=nxi, pressure=pmode, perturb=0.1, seed=4)
    x = M.deformed_state(m, stretch=1.1, shear=0.05, noise=0.02, pressure=-1.3, seed=5)
    ours, ref = str(tmp_path / "ours.exnode"), str(tmp_path / "ref.exnode")
    F.write_exnode(ours, m, x, group="Region")
    R.write_exnode(ref, m, x, group="Region")
    assert os.path.getsize(ref) > 0
    assert open(ours).read() == open(ref).read()


@pytest.mark.parametrize("nxi,pmode", [(3, "node"), (2, "element"), (2, "node"), (3, "element")])
def test_exelem_matches_the_reference_writer(tmp_path, nxi, pmode):
    import build as ob  # oracle/build.py
    if ob.build_ref() is None:
        pytest.skip("the reference tree is not on this machine")
    import fieldexport_ref as R  # oracle/fieldexport_ref.py
    m = M.regular_box(2, 3, 2, nxi_u=nxi, pressure=pmode, perturb=0.1, seed=4)
    x = M.deformed_state(m, stretch=1.1, shear=0.05, noise=0.02, pressure=-1.3, seed=5)
    ours, ref = str(tmp_path / "ours.exelem"), str(tmp_path / "ref.exelem")
    F.write_exelem(ours, m, x, group="Region")
    R.write_exelem(ref, m, x, group="Region")
    assert os.path.getsize(ref) > 0
    assert open(ours).read() == open(ref).read()


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "field_export")


@pytest.mark.parametrize("nxi,pmode", [(3, "node"), (2, "element"), (2, "node"), (3, "element")])
def test_export_matches_the_golden_files(tmp_path, nxi, pmode):
    """The committed golden files (written by the reference's own writer,
    tests/golden/make_field_export_golden.py) against the library's writer,
    on every machine, with or without the reference tree."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_field_export_golden", os.path.join(os.path.dirname(GOLDEN), "make_field_export_golden.py"))
    G = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(G)
    m, x = G.case_state(nxi, pmode)
    base = G.case_name(nxi, pmode)
    F.export(str(tmp_path / base), m, x, group="Region")
    for ext in (".exnode", ".exelem"):
        with open(os.path.join(GOLDEN, base + ext)) as f:
            want = f.read()
        assert open(str(tmp_path / base) + ext).read() == want, base + ext


@pytest.mark.parametrize("nxi,pmode", [(3, "node"), (2, "element")])
def test_export_round_trip(tmp_path, nxi, pmode):
    m = M.regular_box(2, 3, 2, nxi_u=nxi, pressure=pmode, perturb=0.1, seed=4)
    x = M.deformed_state(m, stretch=1.1, shear=0.05, noise=0.02, pressure=-1.3, seed=5)
    node_file, elem_file = F.export(str(tmp_path / "state"), m, x)
    vals = F.read_exnode_values(node_file)
    pnode = set(m.pressure_node_u().tolist()) if pmode == "node" else set()
    for n in range(m.nu):
        v = vals[n + 1]
        assert v[:3] == list(m.X[:, n])
        assert v[3:6] == [x[c * m.nu + n] for c in range(3)]
        assert len(v) == (7 if n in pnode else 6)
    if pmode == "node":
        for q, n in enumerate(m.pressure_node_u()):
            assert vals[n + 1][6] == x[3 * m.nu + q]
    elems = F.read_exelem_nodes(elem_file)
    assert len(elems) == m.ne
    for e in range(m.ne):
        assert elems[e + 1] == list(m.elem_u[e] + 1)
    text = open(elem_file).read()
    assert ("q.Lagrange*q.Lagrange*q.Lagrange" if nxi == 3 else "l.Lagrange*l.Lagrange*l.Lagrange") in text
    assert "coordinate, rectangular cartesian" in open(node_file).read()
