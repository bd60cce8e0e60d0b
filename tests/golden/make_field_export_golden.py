"""Writes the field-export golden files: the exnode and exelem files of four
small states written by the reference's own src/FieldExport.c (compiled
unchanged into oracle/_ref by oracle/build.py and driven the way the
reference's FIELD_IO_NODES_EXPORT / FIELD_IO_ELEMENTS_EXPORT drive it, in
oracle/fieldexport_ref.py).  Needs the reference tree; run from the
repository root:

    python tests/golden/make_field_export_golden.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

CASES = [(3, "node"), (2, "element"), (2, "node"), (3, "element")]


def case_state(nxi, pmode):
    from cm_gb300 import mesh as M
    m = M.regular_box(2, 2, 1, nxi_u=nxi, pressure=pmode, perturb=0.1, seed=4)
    x = M.deformed_state(m, stretch=1.1, shear=0.05, noise=0.02, pressure=-1.3, seed=5)
    return m, x


def case_name(nxi, pmode):
    return "box221_%s_p%s" % ({2: "trilinear", 3: "triquadratic"}[nxi], pmode)


def main():
    import build as ob
    if ob.build_ref() is None:
        raise SystemExit("the reference tree is not on this machine")
    import fieldexport_ref as R
    out = os.path.join(HERE, "field_export")
    os.makedirs(out, exist_ok=True)
    for nxi, pmode in CASES:
        m, x = case_state(nxi, pmode)
        base = os.path.join(out, case_name(nxi, pmode))
        R.write_exnode(base + ".exnode", m, x, group="Region")
        R.write_exelem(base + ".exelem", m, x, group="Region")
        print(base)


if __name__ == "__main__":
    main()
