"""Write the multi-index golden fixture from TSEMLib's own multi-index code.

include/Correspondence.h and include/Multiindex.h compile without AFEPack, deal.II
or LAPACKE, so `make -C oracle ref REF=<checkout>` builds oracle/ref_correspondence.cpp
against them where they lie, into oracle/_ref/.  This script runs that binary and
stores its dump (number -> multi-index, multi-index -> number and the per-degree
ranges of Correspondence<3>, for truncation orders 0..12) as
`multiindex_M12.txt`.  Run in a checkout that has the reference available:

    python tests/golden/make_multiindex_table.py /path/to/TSEMLib
"""
import os
import subprocess
import sys

MAX_M = 12


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_multiindex_table.py <path of the TSEMLib checkout>")
    here = os.path.dirname(os.path.abspath(__file__))
    oracle_dir = os.path.join(os.path.dirname(os.path.dirname(here)), "oracle")
    subprocess.run(["make", "-s", "-C", oracle_dir, "ref", f"REF={os.path.abspath(sys.argv[1])}"], check=True)
    exe = os.path.join(oracle_dir, "_ref", "ref_correspondence")
    out = subprocess.run([exe, str(MAX_M)], check=True, capture_output=True, text=True).stdout
    dst = os.path.join(here, f"multiindex_M{MAX_M}.txt")
    with open(dst, "w") as f:
        f.write(out)
    print("wrote", dst)


if __name__ == "__main__":
    main()
