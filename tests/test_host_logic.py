"""Host-side logic that needs no GPU: the server's batching policy
(tuna_gb300.serve.take_batch), what the server does when no worker can open a
device context, the bench's clock-sample parsing (bench.parse_clock_lines),
whose throttle reasons decide whether a bench number is kept, and the
library's host-side planning (launch shapes, buffer bounds, bin layout)."""
import os
import sys
from collections import deque

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _req(n, key):
    from tuna_gb300.serve import _Req
    return _Req(np.zeros(n, dtype=np.uint8), key, 0.0)


def test_take_batch_groups_by_kind_within_budget():
    from tuna_gb300.serve import take_batch
    a, b, fq = (31, 21, 1, 2**64 - 1, False), (21, 17, 1, 2**64 - 1, False), (31, 21, 1, 2**64 - 1, True)
    q = deque([_req(100, a), _req(50, b), _req(300, a), _req(700, a), _req(10, fq), _req(500, a)])
    batch, rest = take_batch(q, max_bases=1000)
    assert [r.seq.size for r in batch] == [100, 300, 500]  # 700 would pass the budget; 500 still fits
    assert [(r.seq.size, r.key) for r in rest] == [(50, b), (700, a), (10, fq)]
    batch2, rest2 = take_batch(rest, max_bases=10)
    assert [r.seq.size for r in batch2] == [50]  # the oldest goes whatever its size
    assert [r.seq.size for r in rest2] == [700, 10]
    assert take_batch(deque(), 10) == ([], deque())


def test_parse_clock_lines():
    import bench
    ok = "0, 2070, 2070, 900.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n"
    cap = "0, 1980, 2070, 1390.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active\n"
    hot = "0, 1500, 2070, 1200.0, 0x0000000000000040, Not Active, Active, Not Active, Not Active\n"
    out = bench.parse_clock_lines([ok, ok, cap, "garbage\n", "0, [N/A], 2070, 1, 0, a, b, c, d\n"])
    assert out == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    out = bench.parse_clock_lines([hot, ok])
    assert out["reasons"] == ["hw_thermal_slowdown"] and out["sm_mhz"] == (1500.0 + 2070.0) / 2
    assert bench.parse_clock_lines([])["sm_mhz"] is None


def test_server_without_a_device_fails_requests():
    """When no worker can open a device context, waiting requests fail instead
    of waiting forever, and later submits raise (run where there is no GPU)."""
    import time

    import pytest
    import tuna_gb300 as T
    from tuna_gb300 import serve
    if T.library().tg_device_count() > 0:
        pytest.skip("a CUDA device is present: the workers would serve the request")
    seq = np.frombuffer(b"ACGTTGCAAC" * 20, dtype=np.uint8)
    with serve.Server(0, workers=2, max_batch_bases=1 << 20) as srv:
        try:
            f = srv.submit(seq, 31, 21)
        except RuntimeError:  # both workers were already gone
            f = None
        if f is not None:
            with pytest.raises(T.GpuError):
                f.result(timeout=60)
        deadline = time.time() + 60
        while srv._error is None and time.time() < deadline:
            time.sleep(0.02)
        with pytest.raises(RuntimeError, match="no worker could open a device context"):
            srv.submit(seq, 31, 21)


def test_host_planning_invariants(tmp_path):
    """The library's host-side planning (tests/cpp/host_plan_check.cu, linked
    against libtuna_gpu.so, run without a GPU): the phase-1 cut fits in shared
    memory for every (k, m) the GPU path takes, buffer and output size bounds,
    the record-descriptor packing, and the sharing of the 2^20 bins among a
    job's samples (powers of two, contiguous, proportional, segments covering
    each sample's bins)."""
    import shutil
    import subprocess

    import pytest
    import tuna_gb300.build as B
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    lib = B.gpu_lib()
    exe = str(tmp_path / "host_plan_check")
    src = os.path.join(ROOT, "tests", "cpp", "host_plan_check.cu")
    r = subprocess.run([nvcc, *B.ARCH, "-std=c++17", "-O2", "--expt-relaxed-constexpr",
                        "-I", os.path.join(ROOT, "tuna_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                        src, "-o", exe, "-L", os.path.dirname(lib), "-ltuna_gpu",
                        "-Xlinker", "-rpath," + os.path.dirname(lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


def test_server_needs_a_worker():
    import pytest
    from tuna_gb300 import serve
    with pytest.raises(ValueError):
        serve.Server(0, workers=0)


def test_server_result_slabs_recycle_after_last_view():
    """The server's result slabs (tuna_gb300.serve._Pool) go back to the pool
    only when every array viewing them is gone, and are reused by later
    batches that fit (a fake allocator stands in for tg_host_alloc)."""
    import ctypes
    import gc
    import numpy as np
    from tuna_gb300 import serve as S

    class FakeBuffer:
        def __init__(self, n):
            self.buf = (ctypes.c_uint8 * n)()
            self.ptr = ctypes.addressof(self.buf)

        def close(self):
            pass

    class FakeT:
        HostBuffer = FakeBuffer

    pool = S._Pool(FakeT)
    lease = pool.get(1000)
    keys = lease.view(0, 10, np.uint64)
    counts = lease.view(80, 5, np.uint32)
    keys[:] = 3
    del lease
    gc.collect()
    assert not pool._free and int(keys.sum()) == 30
    del keys
    gc.collect()
    assert not pool._free
    del counts
    gc.collect()
    assert len(pool._free) == 1 and pool.allocated == 1
    again = pool.get(600)
    assert not pool._free and pool.allocated == 1
    bigger = pool.get(1 << 21)
    assert pool.allocated == 2
    del again, bigger
