"""The KFF container the library writes around the device-formatted entries
(csrc/host/output.cpp), checked on CPU against the oracle's own KFF writer."""
import pytest


@pytest.mark.parametrize("k", [5, 31, 33, 63])
def test_kff_container_matches_oracle_writer(tmp_path, k):
    """The library's KFF header and footer (csrc/host/output.cpp, driven on CPU
    by tests/cpp/kff_container_check.cpp) are byte for byte the start and the
    end of the oracle's own KFF file for the same k and number of entries (both
    follow the reference's kff_output.hpp calls); the entries in between are the
    device formatter's, checked on the GPU."""
    import os
    import shutil
    import subprocess

    import tuna_gb300.build as B
    from oracle import oracle as O
    if not shutil.which("g++"):
        pytest.skip("g++ not found")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = B.gpu_lib()
    exe = str(tmp_path / "kff_container_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(root, "tuna_gb300", "csrc"),
                        "-I", os.path.join(root, "include"),
                        os.path.join(root, "tests", "cpp", "kff_container_check.cpp"), "-o", exe,
                        "-L", os.path.dirname(lib), "-ltuna_gpu", "-Wl,-rpath," + os.path.dirname(lib)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    seq = b"ACGTTGCAACGGTACCATGCATGGACTAGGCTAGCATCGACTAGCTAGCATCAGGGACTTTACAGCATACGACTAC" * 3
    kff = str(tmp_path / "oracle.kff")
    n = O.write_kff_stream(seq, k, min(21, k - 2), kff)
    assert n > 0
    with open(kff, "rb") as f:
        blob = f.read()
    out = str(tmp_path / "lib")
    subprocess.run([exe, str(k), str(n), out], check=True)
    with open(out + ".head", "rb") as f:
        head = f.read()
    with open(out + ".foot", "rb") as f:
        foot = f.read()
    assert blob.startswith(head) and blob.endswith(foot)
    assert len(blob) == len(head) + n * ((k + 3) // 4 + 4) + len(foot)
