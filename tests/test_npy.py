"""CPU test: the driver's NPY writer (include/euler_operators/euler_npy.hpp)
produces byte-identical files to the reference's own writer
(simulations/save_npy.cpp), whose output is committed as golden files."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

PROG = r"""
#include <euler_npy.hpp>
#include <string>
#include <vector>
int main(int argc, char** argv) {
    std::string dir = argv[1];
    std::vector<double> a(3 * 4 * 5);
    for (int k = 0; k < 5; ++k) for (int j = 0; j < 4; ++j) for (int i = 0; i < 3; ++i)
        a[i + 3 * (j + 4 * k)] = i + 10.0 * j + 100.0 * k + 0.25;
    euler_npy::write_file(dir + "/npy_ours_f64.npy", a.data(), {3, 4, 5}, true);
    std::vector<float> b(12);
    for (std::size_t i = 0; i < b.size(); ++i) b[i] = 0.5f * static_cast<float>(i) - 1.0f;
    euler_npy::write_file(dir + "/npy_ours_f32.npy", b.data(), {2, 3, 2}, true);
    return 0;
}
"""


def test_npy_writer_matches_reference_bytes(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = tmp_path / "w.cpp"
    src.write_text(PROG)
    exe = tmp_path / "w"
    r = subprocess.run(["g++", "-std=c++20", "-O1", f"-I{os.path.join(ROOT, 'include', 'euler_operators')}", str(src),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    subprocess.run([str(exe), str(tmp_path)], check=True)
    for tag in ("f64", "f32"):
        ours = (tmp_path / f"npy_ours_{tag}.npy").read_bytes()
        ref = open(os.path.join(GOLDEN, f"npy_ref_{tag}.npy"), "rb").read()
        assert ours == ref, tag
        arr = np.load(tmp_path / f"npy_ours_{tag}.npy")
        assert arr.flags.f_contiguous
    a = np.load(tmp_path / "npy_ours_f64.npy")
    assert a[1, 2, 3] == 1 + 20 + 300 + 0.25  # (i, j, k) indexing of a layout_left array
