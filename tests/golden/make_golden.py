"""Copies the reference's Mg24 / USDB regression inputs and stored results into
tests/golden/ so that the tests never read the reference tree at run time.

    python tests/golden/make_golden.py /path/to/taurus_vap

Sources (paths inside the reference project):
  int/usdb.sho                                        USDB interaction (ANTOINE)
  examples/gradient_mg24/data/initial_wf.txt          deterministic seed
  examples/gradient_mg24/data/results_vap_benchmark   PNVAP M=5 table
  examples/gradient_mg24/data/results_hfb_benchmark   HFB table
  examples/minima_usdb/data/results_benchmark         USDB minima (random seeds)
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = {
    "int/usdb.sho": "usdb.sho",
    "examples/gradient_mg24/data/initial_wf.txt": "mg24_initial_wf.txt",
    "examples/gradient_mg24/data/results_vap_benchmark": "mg24_results_vap_benchmark",
    "examples/gradient_mg24/data/results_hfb_benchmark": "mg24_results_hfb_benchmark",
    "examples/minima_usdb/data/results_benchmark": "usdb_minima_benchmark",
}

if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference project root>")
    ref = sys.argv[1]
    for src, dst in FILES.items():
        shutil.copyfile(os.path.join(ref, src), os.path.join(HERE, dst))
        print("wrote", dst)
