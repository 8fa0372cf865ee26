"""Copies the reference's shipped cylinder case inputs into
tests/fixtures/cylinder/ as test data: the grid files cylinder05_1.pin and
cylinder05_11122.pin, the plot3d surface cylinder.p3d and the job sheet.
They are input data of the reference (code_mge's cylinder/ directory), kept
here so that the tests that read them run where the reference tree is not
present.  Run from the repository root with the reference tree's cylinder/
directory as the argument."""
import os
import shutil
import sys

FILES = ("cylinder05_1.pin", "cylinder05_11122.pin", "cylinder.p3d", "jobsheet")


def main(src):
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cylinder")
    os.makedirs(dst, exist_ok=True)
    for f in FILES:
        shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
        print("copied", f)


if __name__ == "__main__":
    main(sys.argv[1])
