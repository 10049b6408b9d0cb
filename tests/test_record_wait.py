"""The bounded wait of the stage kernel's chunk reduction (stage.cuh,
sum_polled_records).

In the one-wave stage instance the chunks of a sink tile store their partial
records with no fence; the CTA that counts last re-reads a record until its
store has landed.  A record slot holds an empty pattern until then.  These
tests drive sum_polled_records directly from a one-thread kernel compiled
from the library's own header:

  * landed records are summed in chunk order (double-single for the float2
    records of the FP32 modes, FP64 otherwise), bit-identical to the same
    sums on the host, and every slot is emptied for the next launch;
  * a record that never lands (a slot nothing writes) ends the wait after its
    read limit, about a second: the sum is NaN, the call reports failure and
    the slots are emptied, so the kernel returns and the context stays usable.
    The stage kernel turns that failure into RED_ERR_TIMEOUT on the system.
"""
import ctypes as C
import math
import os
import subprocess
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "red.cuda_gb300", "csrc")
EMPTY = 0x7ff0000000000001

SHIM = r'''
#include "stage.cuh"
using namespace redgb;

template <typename T>
__global__ void k_sum(unsigned long long* recs, int n, T* out, int* ok)
{
    T s = T();
    *ok = sum_polled_records(recs, 1, 0, n, s) ? 1 : 0;
    *out = s;
}

// recs: n 8-byte slots in and out; out: 2 floats or 1 double; returns a CUDA error code
extern "C" int run_sum(int fp64, unsigned long long* recs, int n, void* out, int* ok)
{
    unsigned long long* d_recs = nullptr;
    void* d_out = nullptr;
    int* d_ok = nullptr;
    cudaMalloc(&d_recs, n * 8);
    cudaMalloc(&d_out, 8);
    cudaMalloc(&d_ok, sizeof(int));
    cudaMemcpy(d_recs, recs, n * 8, cudaMemcpyHostToDevice);
    if (fp64) k_sum<<<1, 1>>>(d_recs, n, (double*)d_out, d_ok);
    else k_sum<<<1, 1>>>(d_recs, n, (float2*)d_out, d_ok);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) {
        cudaMemcpy(recs, d_recs, n * 8, cudaMemcpyDeviceToHost);
        cudaMemcpy(out, d_out, 8, cudaMemcpyDeviceToHost);
        e = cudaMemcpy(ok, d_ok, sizeof(int), cudaMemcpyDeviceToHost);
    }
    cudaFree(d_recs);
    cudaFree(d_out);
    cudaFree(d_ok);
    return (int)e;
}
'''


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    d = tmp_path_factory.mktemp("recwait")
    src = d / "shim.cu"
    src.write_text(SHIM)
    so = d / "shim.so"
    nvcc = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
    subprocess.check_call([nvcc, "-shared", "-Xcompiler", "-fPIC", "-gencode", "arch=compute_103a,code=sm_103a",
                           "-O3", "-std=c++17", "--expt-relaxed-constexpr", "-ftz=true",
                           "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-o", str(so), str(src)])
    L = C.CDLL(str(so))
    L.run_sum.restype = C.c_int
    L.run_sum.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_int)]
    return L


def run(shim, fp64, words):
    recs = np.array(words, dtype=np.uint64)
    out = np.zeros(1, dtype=np.float64) if fp64 else np.zeros(2, dtype=np.float32)
    ok = C.c_int(-1)
    t0 = time.perf_counter()
    rc = shim.run_sum(1 if fp64 else 0, recs.ctypes.data, len(recs), out.ctypes.data, C.byref(ok))
    assert rc == 0, rc
    return recs, out, ok.value, time.perf_counter() - t0


def f2_word(hi, lo):
    return int(np.array([hi, lo], dtype=np.float32).view(np.uint64)[0])


def ds_add_host(a, b):
    """dsn_add of common.cuh restated in float32 (TwoSum of the high parts,
    the low parts added to its error, one fast renormalisation), for the
    expected bits."""
    f = np.float32
    s = f(a[0] + b[0])
    bb = f(s - a[0])
    e = f(f(a[0] - f(s - bb)) + f(b[0] - bb))
    e = f(e + f(a[1] + b[1]))
    hi = f(s + e)
    return (hi, f(e - f(hi - s)))


def test_landed_records_sum_in_order_and_empty_their_slots(shim):
    rng = np.random.default_rng(7)
    n = 37                                    # more than two batches of 16
    vals = rng.normal(size=n) * 1e-6
    recs, out, ok, _ = run(shim, True, [int(np.float64(v).view(np.uint64)) for v in vals])
    assert ok == 1
    acc = 0.0
    for v in vals:
        acc += v
    assert out[0] == acc
    assert np.all(recs == EMPTY)
    hi = rng.normal(size=n).astype(np.float32)
    lo = (hi * np.float32(1e-8)).astype(np.float32)
    recs, out, ok, _ = run(shim, False, [f2_word(h, l) for h, l in zip(hi, lo)])
    assert ok == 1 and np.all(recs == EMPTY)
    assert np.all(np.isfinite(out))
    ref = (np.float32(0), np.float32(0))
    for h, l in zip(hi, lo):
        ref = ds_add_host(ref, (h, l))
    assert out[0] == ref[0] and out[1] == ref[1]


@pytest.mark.parametrize("fp64", [True, False])
def test_a_record_that_never_lands_ends_the_wait(shim, fp64):
    words = [int(np.float64(1.0).view(np.uint64)) if fp64 else f2_word(1.0, 0.0)] * 5
    words[3] = EMPTY                          # a slot nothing writes
    recs, out, ok, secs = run(shim, fp64, words)
    assert ok == 0
    assert all(math.isnan(float(x)) for x in np.atleast_1d(out)[:1])
    assert np.all(recs == EMPTY)
    assert secs < 30.0
    # the context is still usable: a landed set sums right after
    recs, out, ok, _ = run(shim, fp64, [words[0]] * 4)
    assert ok == 1 and float(out[0]) == 4.0

