"""Copy the FESOM2 mesh folders the reference's tests carry (Soufflet channel, the PI mesh and
PI with ice-shelf cavities, tests/data/MESHES/{soufflet,pi,pi_cavity}) into
tests/golden/mesh_*.npz, as the raw arrays
of their .out files, so that tests can build those meshes where the reference tree is
absent.  Run from the repository root:  python tests/golden/make_mesh_fixtures.py [ref]
(ref: the reference checkout; default: the FESOM2_REFERENCE environment variable).
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from fesom2_gb300 import meshio as MI  # noqa: E402


def main(ref: str = "") -> None:
    ref = ref or os.environ.get("FESOM2_REFERENCE", "")
    if not ref:
        raise SystemExit("give the reference checkout as an argument or in FESOM2_REFERENCE")
    for name in ("soufflet", "pi", "pi_cavity"):
        r = MI.read_files(os.path.join(ref, "tests", "data", "MESHES", name))
        out = os.path.join(ROOT, "tests", "golden", f"mesh_{name}.npz")
        MI.save_files(r, out)
        print(out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main(*sys.argv[1:])
