"""Copy the reference's own test fixtures (golden vectors) into tests/golden/.

The reference ships three end-to-end fixtures under tests/ of its source tree:
assembled/lap16x16, assembled/lap4x4 and elemental/e4x4.  They are data
(matrices, right-hand sides, direct-solve solutions and control files), not
source code.  The GPU test box has no copy of the reference, so this script
copies them here once, byte for byte, and records their SHA-256 in
MANIFEST.txt.  Run from this container:  python tests/golden/make_golden.py
"""
import hashlib
import os
import shutil
import sys

SRC = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/tests"
HERE = os.path.dirname(os.path.abspath(__file__))
CASES = {
    "lap16x16": ("assembled/lap16x16", ["DOUG.ctl", "Lap16x16.txt", "rhs.xdr", "csolution.xdr"]),
    "lap4x4": ("assembled/lap4x4", ["DOUG.ctl", "Lap4x4.txt", "rhs.dat", "solution_correct.dat"]),
    "e4x4": ("elemental/e4x4", ["DOUG.ctl", "doug_info.dat", "doug_element.dat", "doug_system.dat",
                                "doug_coord.dat", "doug_freemap.dat", "csolution.xdr",
                                "doug_csolution.dat"]),
}


def main():
    lines = []
    for name, (sub, files) in CASES.items():
        dst = os.path.join(HERE, name)
        os.makedirs(dst, exist_ok=True)
        for f in files:
            s = os.path.join(SRC, sub, f)
            d = os.path.join(dst, f)
            shutil.copyfile(s, d)
            os.chmod(d, 0o644)
            h = hashlib.sha256(open(d, "rb").read()).hexdigest()
            lines.append(f"{h}  {name}/{f}  (reference tests/{sub}/{f})")
    with open(os.path.join(HERE, "MANIFEST.txt"), "w") as fh:
        fh.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
