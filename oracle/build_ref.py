"""Build the reference-side checker and regenerate the golden vectors.

Compiles oracle/ref_kat.cpp against the reference's own vendored headers
(external/pcg-cpp-0.98/include, external/eigen) into oracle/_ref/ref_kat, runs
it, and writes tests/golden/ref_kat.json.  Only this script reads the
reference tree, and only where it exists (the build container); the fixture
it writes is committed so that tests elsewhere need no reference.

The reference tree is taken from --reference, else from the environment
variable BTE_REFERENCE_TREE, else from the build container's mount point.

Usage: python oracle/build_ref.py [--reference DIR] [--no-write]
"""
import argparse
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


_MOUNT = "/root/reference"  # where the build container mounts the reference


def reference_tree():
    """The reference tree to build from, or None where it does not exist."""
    path = os.environ.get("BTE_REFERENCE_TREE", _MOUNT)
    return path if os.path.isdir(path) else None


def build(reference: str) -> str:
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "ref_kat")
    cmd = [
        "g++", "-std=c++17", "-O2", "-ffp-contract=off",
        "-I", os.path.join(reference, "external", "pcg-cpp-0.98", "include"),
        "-I", os.path.join(reference, "external", "eigen"),
        os.path.join(HERE, "ref_kat.cpp"), "-o", exe,
    ]
    subprocess.run(cmd, check=True)
    return exe


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    ap.add_argument("--no-write", action="store_true")
    args = ap.parse_args()
    if args.reference is None:
        args.reference = reference_tree()
    if not args.reference or not os.path.isdir(args.reference):
        print(f"reference tree {args.reference} absent; nothing to build")
        return 0
    exe = build(args.reference)
    text = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    data = json.loads(text)
    if not args.no_write:
        path = os.path.join(REPO, "tests", "golden", "ref_kat.json")
        with open(path, "w") as f:
            json.dump(data, f, indent=1)
        print("wrote", path)
    return 0


if __name__ == "__main__":
    sys.exit(main())
