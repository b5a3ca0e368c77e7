"""The NPY writer behind the result tree (epic2d_output.hpp, the HDF5-free
counterpart of src/output.cpp): files it writes load in numpy with the shape,
dtype and element order given."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include "epic2d_output.hpp"
int main(int argc, char** argv) {
  std::filesystem::path d = argv[1];
  std::vector<double> a(7 * 3);
  for (size_t k = 0; k < a.size(); k++) a[k] = 0.5 * k - 3.25;
  epic2d::write_npy(d / "a.npy", a.data(), {7, 3});
  epic2d::write_npy(d / "b.npy", a.data(), {5});
  epic2d::write_npy(d / "c.npy", a.data(), {0, 2});
  std::vector<double> big(123456);
  for (size_t k = 0; k < big.size(); k++) big[k] = 1.0 / (k + 1);
  epic2d::write_npy(d / "d.npy", big.data(), {123456, 1});
  return 0;
}
"""


def test_npy_writer_round_trip(tmp_path):
    src = tmp_path / "w.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "w"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "epic2d_mcc_gb300", "host"), str(src), "-o", str(exe)], check=True)
    subprocess.run([str(exe), str(tmp_path)], check=True)
    a = np.load(tmp_path / "a.npy")
    assert a.dtype == np.float64 and a.shape == (7, 3)
    assert np.array_equal(a.reshape(-1), 0.5 * np.arange(21) - 3.25)
    b = np.load(tmp_path / "b.npy")
    assert b.shape == (5,) and np.array_equal(b, 0.5 * np.arange(5) - 3.25)
    assert np.load(tmp_path / "c.npy").shape == (0, 2)
    d = np.load(tmp_path / "d.npy")
    assert d.shape == (123456, 1) and np.array_equal(d[:, 0], 1.0 / (np.arange(123456) + 1))
    for name in "abcd":
        raw = (tmp_path / (name + ".npy")).read_bytes()
        header_len = raw[8] | (raw[9] << 8)
        assert (10 + header_len) % 64 == 0
