"""P files written by the compiled reference (oracle/_ref, the unmodified sources) with
load_affinities = 2 (src/tsne.cpp:333-366): P_row.dat, P_col.dat and P_val.dat of the
1,000-point end-to-end problem of fitsne_golden.npz (e2e_X, perplexity 15, VP-tree kNN),
stored as arrays; the test writes them back to files for the library to load.

    python tests/golden/make_pfiles.py   (needs the reference tree: make -C oracle ref)
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))


def main():
    import oracle
    oracle.build_reference()
    ref = oracle.Reference()
    g = np.load(os.path.join(HERE, "fitsne_golden.npz"))
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            ref.run(g["e2e_X"], g["e2e_Y0"], no_dims=2, perplexity=15.0, max_iter=1, stop_lying_iter=100,
                    mom_switch_iter=100, learning_rate=200.0, nthreads=1, load_affinities=2)
            out = {"P_row": np.fromfile("P_row.dat", np.uint32), "P_col": np.fromfile("P_col.dat", np.uint32),
                   "P_val": np.fromfile("P_val.dat", np.float64)}
        finally:
            os.chdir(cwd)
    np.savez_compressed(os.path.join(HERE, "pfiles_e2e.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
