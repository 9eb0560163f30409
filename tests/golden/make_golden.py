"""Generate the golden fixtures under tests/golden/ from the reference's own code.

Run in a container where the reference is mounted (it is not needed at test
time):  python tests/golden/make_golden.py /path/to/BladeMaster-Lab

Only the reference modules that import without Warp are used:
``blademaster_warp/geometry.py`` (points, stencil) and
``blademaster_warp/topology.py`` (compatible, components).  Each fixture is
a small .npz with the inputs and the reference's outputs.
"""

import sys
from pathlib import Path
import numpy as np

HERE = Path(__file__).resolve().parent


def main(reference_root):
    sys.path.insert(0, str(reference_root))
    from blademaster_warp.geometry import points, stencil
    from blademaster_warp.topology import components, compatible

    cases = {
        # name: (size, spacing, shape, seed)
        "default_block": ((0.06, 0.03, 0.03), 0.0075, "block", 0),
        "freefall_block": ((0.14, 0.10, 0.08), 0.01, "block", 0),
        "jitter_block": ((0.06, 0.03, 0.03), 0.006, "block", 1),
        "banana": ((0.12, 0.06, 0.03), 0.006, "banana", 0),
        "cylinder": ((0.036, 0.036, 0.12), 0.006, "cylinder", 0),
        "odd_spacing": ((0.03, 0.03, 0.03), 0.007, "block", 2),
    }
    for name, (size, spacing, shape, seed) in cases.items():
        x, origin, cells = points(size, spacing, shape, seed)
        nodes, w, g = stencil(x, origin, spacing, cells)
        np.savez_compressed(
            HERE / f"geometry_{name}.npz",
            size=np.asarray(size),
            spacing=spacing,
            shape=shape,
            seed=seed,
            x=x,
            origin=origin,
            cells=cells,
            nodes=nodes,
            weights=w,
            gradients=g,
        )
    # Piece counting: the default block cut by random planes.
    rng = np.random.default_rng(11)
    x, origin, cells = points((0.06, 0.03, 0.03), 0.0075, "block", 0)
    nodes, w, _ = stencil(x, origin, 0.0075, cells)
    code_sets = {
        "uncut": np.zeros(len(x), np.int64),
        "one_cut": np.where(x[:, 0] < 0, 1, 2).astype(np.int64),
        "partial_cut": np.where(x[:, 2] > 0.012, np.where(x[:, 0] < 0, 1, 2), 0).astype(np.int64),
        "two_cuts": (np.where(x[:, 0] < -0.01, 1, 2) + 3 * np.where(x[:, 0] < 0.015, 1, 2)).astype(np.int64),
        "random27": rng.integers(0, 27, len(x)).astype(np.int64),
    }
    labels = {}
    for key, codes in code_sets.items():
        lab, sizes = components(nodes, w, codes)
        labels[f"{key}_codes"] = codes
        labels[f"{key}_labels"] = lab
        labels[f"{key}_sizes"] = sizes
    pairs = rng.integers(0, 3**6, (400, 2))
    labels["compat_pairs"] = pairs
    labels["compat_values"] = np.array([compatible(a, b) for a, b in pairs])
    np.savez_compressed(HERE / "topology_default_block.npz", nodes=nodes, weights=w, **labels)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/BladeMaster-Lab")
    main(sys.argv[1])
