"""Regenerates the golden fixtures in this folder from the reference checkout.

Usage: python tests/golden/make_golden.py /path/to/rtbvh-reference

* teapot_tris.npy -- the triangles the reference's tests load from
  objects/teapot.obj (src/lib.rs:194-244 de-indexes the OBJ faces in file
  order with l3d). float32, shape (6320, 3, 3).
* known_answers.json -- the literal expected values of the reference's own
  unit tests for the BVH path, each with the file:line it comes from.

Run once in a container that has the reference checkout; the outputs are
committed so that the tests never need the reference at run time.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_obj_triangles(path):
    verts = []
    tris = []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if not parts:
                continue
            if parts[0] == "v":
                verts.append([float(x) for x in parts[1:4]])
            elif parts[0] == "f":
                idx = [int(p.split("/")[0]) for p in parts[1:]]
                idx = [i - 1 if i > 0 else len(verts) + i for i in idx]
                for k in range(1, len(idx) - 1):  # fan triangulation (the teapot is all triangles)
                    tris.append([verts[idx[0]], verts[idx[k]], verts[idx[k + 1]]])
    return np.asarray(tris, dtype=np.float32)


def main(ref_root):
    tris = load_obj_triangles(os.path.join(ref_root, "objects", "teapot.obj"))
    assert tris.shape == (6320, 3, 3), tris.shape
    np.save(os.path.join(HERE, "teapot_tris.npy"), tris)
    known = {
        "morton_split": {"source": "src/morton.rs:109-115", "cases": [[2, 8], [4, 64], [8, 512], [32, 32768]]},
        "prefix_sum": {"source": "src/utils.rs:295-345", "input": [1, 2, 3, 4, 5, 6],
                       "output": [1, 3, 6, 10, 15, 21], "zero_count_returns_first": 1},
        "abi_sizes": {"source": "rtbvh_ffi/src/lib.rs:855-866", "RTAabb": 32, "RTBvhNode": 32, "RTMbvhNode": 128},
        "result_codes": {"source": "rtbvh_ffi/src/lib.rs:17-25",
                         "Ok": 0, "Error": 1, "NoPrimitives": 2, "InequalAabbsAndPrimitives": 3, "Nan": 4},
        "bvh_type": {"source": "rtbvh_ffi/src/lib.rs:129-133", "LocallyOrderedClustered": 0, "BinnedSAH": 1},
        "quad_hit": {"source": "rtbvh_ffi/src/lib.rs:945-1019",
                     "vertices": [[-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, -1, 1], [1, 1, 1], [-1, 1, 1]],
                     "origin": [0, 0, 0], "direction": [0, 0, 1], "t_in": 1e26, "t_expected": 1.0,
                     "callback_t_min": 1e-5},
        "five_triangles": {"source": "src/lib.rs:246-311", "leaf_sizes": list(range(1, 11)),
                           "triangles": [
                               [[128.79, -1422.82, 0.16], [128.5, -1426.88, 0.16], [128.79, -1426.9067, 0.16]],
                               [[129.8, -1422.8629, 0.16], [128.79, -1422.82, 0.16], [128.79, -1426.9067, 0.16]],
                               [[129.8, -1422.8629, 0.16], [128.79, -1426.9067, 0.16], [129.8, -1427.0, 0.16]],
                               [[130.2, -1422.88, 0.16], [129.8, -1422.8629, 0.16], [129.8, -1427.0, 0.16]],
                               [[130.2, -1422.88, 0.16], [129.8, -1427.0, 0.16], [130.2, -1423.13, 0.16]]]},
        "two_triangle_quad": {"source": "src/lib.rs:66-124",
                              "vertices": [[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]],
                              "triangles": [[0, 1, 2], [0, 2, 3]]},
        "teapot_structure": {"source": "src/builders/binned_sah.rs:407-458, src/builders/locb.rs:336-388",
                             "prim_count": 6320,
                             "checks": ["n <= nodes <= 2n", "root bounds valid", "validate()",
                                        "root bounds strictly contain every vertex"]},
    }
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(known, f, indent=1)
    print("wrote", tris.shape)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/rtbvh-reference")
    main(sys.argv[1])
