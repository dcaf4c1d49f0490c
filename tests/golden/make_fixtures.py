"""Collect the reference's own golden data into tests/golden/ (run once, in a
checkout that has the zosimos sources; the GPU machine never runs this).

* the two input images of lib/zosimos/tests/input/ (RGBA8 PNGs), and
* the blockhash256 goldens of lib/zosimos/tests/reference/*.crc.png (hex text).

Usage:  python tests/golden/make_fixtures.py /path/to/zosimos
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(root: str) -> None:
    base = os.path.join(root, "lib", "zosimos", "tests")
    for name in ("background.png", "foreground.png"):
        shutil.copyfile(os.path.join(base, "input", name), os.path.join(HERE, name))
    hashes = {}
    for name in sorted(os.listdir(os.path.join(base, "reference"))):
        with open(os.path.join(base, "reference", name)) as f:
            hashes[name.replace(".crc.png", "")] = [ln.strip() for ln in f if ln.strip()]
    with open(os.path.join(HERE, "blockhash_goldens.txt"), "w") as f:
        f.write("# name: accepted blockhash256 values (lib/zosimos/tests/reference/<name>.crc.png)\n")
        for k, v in hashes.items():
            f.write(f"{k}: {' '.join(v)}\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py /path/to/zosimos")
    main(sys.argv[1])
