"""Build the golden fixtures under tests/golden/.

1. Copies the reference crate's own FP64 outputs (written by its integration
   tests ``tests/harmonic_tests.rs`` and ``tests/ground_state_tests.rs``) from a
   checkout of Wleter/split_operator: ``<ref>/tests/test_data/*.npy``.
2. Writes ``fft_known_answer.npz``: the 4x4 known answer of the reference's
   ``tests/fft_tests.rs:11-78`` as arrays (input, forward result).

Usage: python tests/golden/make_golden.py /path/to/split_operator
"""
import shutil
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
COPIED = [
    "harmonic.npy", "harmonic_potential.npy", "harmonic_space_grid.npy", "harmonic_time.npy",
    "harmonic_imaginary.npy", "harmonic_imaginary_potential.npy",
    "harmonic_imaginary_space_grid.npy", "harmonic_imaginary_time.npy",
    "lj_ground_space.npy", "lj_ground_space_potential.npy",
    "lj_ground_space_space_grid.npy", "lj_ground_space_time.npy",
]


def main(ref_root: str) -> None:
    src = Path(ref_root) / "tests" / "test_data"
    for name in COPIED:
        shutil.copyfile(src / name, HERE / name)
    # tests/fft_tests.rs:14-39 (input) and :49-74 (expected forward transform along axis 0)
    inp = np.arange(1, 17, dtype=np.float64).reshape(4, 4).astype(np.complex128)
    fwd = np.array([[14, 16, 18, 20],
                    [-4 + 4j] * 4,
                    [-4] * 4,
                    [-4 - 4j] * 4], dtype=np.complex128)
    np.savez(HERE / "fft_known_answer.npz", input=inp, forward=fwd)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the split_operator crate checkout>")
    main(sys.argv[1])
