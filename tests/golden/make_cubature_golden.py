"""Write tests/golden/cubature_ref.json from HyperFox's own Cubature class.

oracle/build_ref.sh compiles the reference's src/element/Cubature.cpp (with
ErrorHandle.cpp and a small shim) into oracle/_ref/libref_cubature.so; this
script runs it for every simplex rule the HDG path uses (dims 1-3, orders
1..10) and stores the points and weights, so the tests can check the tables
on machines without the HyperFox source tree.
"""
import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_cubature.so"))
    f = lib.ref_cubature
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    out = {}
    for dim in (1, 2, 3):
        for order in range(1, 11):
            X = np.zeros(400)
            W = np.zeros(200)
            n = f(dim, order, 0, X.ctypes.data, W.ctypes.data, 200)
            assert n > 0, (dim, order, n)
            out["%d_%d" % (dim, order)] = {"points": X[:n * dim].tolist(), "weights": W[:n].tolist()}
    with open(os.path.join(HERE, "cubature_ref.json"), "w") as fh:
        json.dump(out, fh)


if __name__ == "__main__":
    main()
