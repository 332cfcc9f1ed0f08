"""The C++ front end (include/hmpc_gb300/hmpc.hpp): a C++ program written
against the hmpc::comp::queue / hmpc::expr names is compiled, run on the GPU,
and its results are compared with the oracle."""
import pathlib
import shutil
import subprocess

import numpy as np
import pytest

from hmpc_gb300 import _lib

pytestmark = pytest.mark.gpu
ROOT = pathlib.Path(__file__).resolve().parents[1]
Q_256 = 0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001
KEY = [1, 2, 3, 4, 5, 6, 7, 8]


def test_cpp_frontend(tmp_path, oracle):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("needs g++")
    exe = tmp_path / "frontend_test"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(ROOT / "tests/cpp/frontend_test.cpp"),
                    "-L", str(_lib.LIB_PATH.parent), "-lhmpc_gb300", f"-Wl,-rpath,{_lib.LIB_PATH.parent}", "-o",
                    str(exe)], check=True)
    run = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    n, batch = 1024, 3
    m = oracle.Modulus(Q_256)
    load = lambda name: np.fromfile(tmp_path / name, dtype=np.uint32).reshape(m.limbs, -1)  # noqa: E731
    x = np.zeros((m.limbs, n * batch), dtype=np.uint32)
    x[0] = np.arange(1, n * batch + 1, dtype=np.uint32)
    assert np.array_equal(load("ntt.bin"), oracle.ntt(m, n, batch, src=x))
    u = oracle.ntt(m, n, batch, sampler="cbd", variance_x2=1, key=KEY, nonce=[0, 0, 0])
    v = oracle.ntt(m, n, batch, sampler="cbd", variance_x2=20, key=KEY, nonce=[n * batch, 0, 0])
    assert np.array_equal(load("u.bin"), u)
    assert np.array_equal(load("v.bin"), v)
    a = x.reshape(-1)[: n * m.limbs].reshape(m.limbs, n)  # the C++ test uploads the first n*L host words
    au = oracle.binary(m, oracle.OP_MUL, a, u, elements=n * batch)
    w = oracle.ntt(m, n, batch, src=oracle.binary(m, oracle.OP_ADD, au, v), inverse=True)
    assert np.array_equal(load("w.bin"), w)
    y = load("ntt.bin")
    mat = np.zeros((m.limbs, 2 * batch * n), dtype=np.uint32)
    mat[0] = 3 * np.arange(2 * batch * n, dtype=np.uint32) + 7
    assert np.array_equal(load("matvec.bin"), oracle.matvec(m, 1, 2, batch, n, mat, y))
    assert np.array_equal(load("sum.bin")[:, 0], oracle.reduce_mod(m, "add", y))
    assert np.array_equal(load("product.bin")[:, 0], oracle.reduce_mod(m, "multiply", y))
