"""Copy the reference's hypercam golden vectors into tests/golden/hypercam/.

The reference ships one external golden vector for the render chain:
``crates/optics-inverse/tests/data/hypercam/{forward.npy, thickness.npy,
meta.txt}`` (used by ``crates/optics-inverse/tests/hypercam_forward.rs``).
The GPU machine has no copy of the reference, so the files are committed here
unchanged; this script re-creates them and prints their SHA-256.

Usage: python tests/golden/make_hypercam.py [REFERENCE_ROOT]
"""

import hashlib
import pathlib
import shutil
import sys

ref = pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
src = ref / "crates/optics-inverse/tests/data/hypercam"
dst = pathlib.Path(__file__).resolve().parent / "hypercam"
dst.mkdir(parents=True, exist_ok=True)
for name in ("forward.npy", "thickness.npy", "meta.txt"):
    shutil.copyfile(src / name, dst / name)
    print(name, hashlib.sha256((dst / name).read_bytes()).hexdigest())
