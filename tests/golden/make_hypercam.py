"""Copy the reference's hypercam golden vectors into tests/golden/hypercam/.

The reference ships one external golden vector for the render chain:
``crates/optics-inverse/tests/data/hypercam/{forward.npy, thickness.npy,
meta.txt}`` (used by ``crates/optics-inverse/tests/hypercam_forward.rs``).
The GPU machine has no copy of the reference, so the files are committed here
unchanged; this script re-creates them and prints their SHA-256.

Usage: python tests/golden/make_hypercam.py REFERENCE_ROOT
       (or OPTICS_STUDIO_REFERENCE=REFERENCE_ROOT python tests/golden/make_hypercam.py)
REFERENCE_ROOT is the root of an optics-studio checkout.
"""

import hashlib
import os
import pathlib
import shutil
import sys

root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("OPTICS_STUDIO_REFERENCE")
if not root:
    sys.exit(__doc__)
ref = pathlib.Path(root)
src = ref / "crates/optics-inverse/tests/data/hypercam"
dst = pathlib.Path(__file__).resolve().parent / "hypercam"
dst.mkdir(parents=True, exist_ok=True)
for name in ("forward.npy", "thickness.npy", "meta.txt"):
    shutil.copyfile(src / name, dst / name)
    print(name, hashlib.sha256((dst / name).read_bytes()).hexdigest())
