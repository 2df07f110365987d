"""The chunk plan of the host-resident step (csrc/fd_host_plan.h, used by
fd_fused_step_packed_host), compiled with the host C++ compiler and checked
without a GPU: the chunks tile the strips, the ramp and the cap on the chunk
count hold, the compute order visits every chunk once, and every chunk's
compute waits for the uploads of all rows it reads, wrap-around included."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include "fd_host_plan.h"
int main(int argc, char** argv) {
  const fd::HostPlan p = fd::host_plan(std::atoi(argv[1]), std::atoi(argv[2]));
  std::printf("%d %d\n", p.R, p.nstrips);
  for (int v : p.cb) std::printf("%d ", v);
  std::printf("\n");
  for (int v : p.order) std::printf("%d ", v);
  std::printf("\n");
  for (int v : p.need) std::printf("%d ", v);
  std::printf("\n");
  return 0;
}
"""


@pytest.fixture(scope="module")
def plan_exe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("plan")
    src, exe = d / "plan.cpp", d / "plan"
    src.write_text(DRIVER)
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(REPO, "fingering_dynamics_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    return str(exe)


def plan(exe, H, chunk_rows):
    out = subprocess.run([exe, str(H), str(chunk_rows)], capture_output=True, text=True, check=True).stdout
    lines = out.strip().split("\n")
    R, nstrips = map(int, lines[0].split())
    return R, nstrips, [list(map(int, ln.split())) for ln in lines[1:]]


CASES = [(3, 0), (15, 0), (16, 0), (17, 0), (33, 0), (75, 0), (130, 7), (1000, 0), (2048, 0), (2048, 64),
         (2048, 16), (4097, 0), (16384, 16), (65536, 0), (65536, 16)]


@pytest.mark.parametrize("H,chunk_rows", CASES)
def test_host_plan(plan_exe, H, chunk_rows):
    R, nstrips, (cb, order, need) = plan(plan_exe, H, chunk_rows)
    assert R == min(16, H) and nstrips == -(-H // R)
    K = len(cb) - 1
    assert cb[0] == 0 and cb[-1] == nstrips and all(a < b for a, b in zip(cb, cb[1:]))
    assert 1 <= K <= 256
    rows = [(cb[c] * R, min(cb[c + 1] * R, H)) for c in range(K)]
    # every chunk but the last holds at least two rows (its neighbours' halo rows lie in adjacent chunks)
    assert all(r1 - r0 >= 2 for r0, r1 in rows[:-1])
    # the ramp: the first chunks are 1, 1, 2, 4 strips (at most the middle chunk size)
    sizes = [b - a for a, b in zip(cb, cb[1:])]
    m = max(sizes) if sizes else 1
    for k, want in enumerate((1, 1, 2, 4)[:K - 1]):
        assert sizes[k] == min(want, m)
    assert sorted(order) == list(range(K))

    def chunk_of(row):
        return next(c for c, (r0, r1) in enumerate(rows) if r0 <= row < r1)

    for c in range(K):
        r0, r1 = rows[c]
        read = {chunk_of(y % H) for y in range(r0 - 2, r1 + 2)}
        assert max(read) <= need[c], (c, sorted(read), need[c])
