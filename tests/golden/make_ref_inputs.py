"""Copy the reference's example inputs into tests/golden/ref_inputs/.

The QS-Cube/ED source tree ships example input sets (input_ex1 .. input_ex5)
but no outputs.  Their input.dat namelists and list_* files are the only
reference-held inputs for the hot path, so the GPU parity tests read them
(through ed_gb300.inputs) and compare the GPU library with the oracle on
them.  The reference tree is not present where the GPU tests run, so the
files are committed here; this script regenerates them:

    python tests/golden/make_ref_inputs.py [REFERENCE_ROOT]

Files copied (paths within the reference tree):
  input_ex1/input.dat, list_xxz_term_36.dat, list_cf_ss.dat,
            list_local_mag.dat, list_site_position_36_type1.dat
            (6x6 lattice, NOD=3, 72 bonds, ALG=2 TRLan, DSF spsmsz=3)
  input_ex2/input.dat   (ex1's lattice with ALG=3)
  input_ex3/input.dat, list_xxz_term_1000.dat, list_site_position_1000_type1.dat
            (10x10x10 cubic lattice, NOD=2, 3000 bonds, ALG=1, DSF q=(0,0,pi/2))
  input_ex5/input.dat, list_xxz_term_36.dat
            (6x6 triangular lattice, NOD=3, 108 bonds, ALG=1)
Nothing is edited: the files are byte copies.
"""
import os
import shutil
import sys

FILES = {
    "input_ex1": ["input.dat", "list_xxz_term_36.dat", "list_cf_ss.dat", "list_local_mag.dat",
                  "list_site_position_36_type1.dat"],
    "input_ex2": ["input.dat"],
    "input_ex3": ["input.dat", "list_xxz_term_1000.dat", "list_site_position_1000_type1.dat"],
    "input_ex5": ["input.dat", "list_xxz_term_36.dat"],
}


def main(ref_root: str = "/root/reference") -> None:
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_inputs")
    for d, names in FILES.items():
        os.makedirs(os.path.join(out, d), exist_ok=True)
        for n in names:
            shutil.copyfile(os.path.join(ref_root, d, n), os.path.join(out, d, n))
    print(f"copied into {out}")


if __name__ == "__main__":
    main(*sys.argv[1:2])
