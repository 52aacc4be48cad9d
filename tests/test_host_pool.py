"""The host worker pool of a context (relaibilitygpu_gb300/csrc/nr_pool.h).

A batch call runs several short jobs on the pool back to back.  The stress program below runs
jobs of many sizes, helper counts and grab sizes one after another, with idle gaps that let the
workers go to sleep, and checks that every index of every job ran exactly once before the job
returned -- the property a late worker claiming into the next job broke in an earlier layout of
the pool's job word.  It is built plainly and, where the compiler has it, under ThreadSanitizer."""
import os
import shutil
import subprocess

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "relaibilitygpu_gb300", "csrc")

STRESS = r"""
#include "nr_pool.h"
#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char **argv)
{
    const int jobs = argc > 1 ? atoi(argv[1]) : 2000;
    for (int workers : {1, 3, 7}) {
        NrPool pool(workers);
        for (int it = 0; it < jobs; ++it) {
            const int n = 1 + (it * 7919) % 3000;
            std::vector<int> hit(n, 0);
            std::function<void(int)> fn = [&](int i) { hit[i]++; };
            pool.run(n, it % (workers + 1), 1 + it % 40, fn);
            for (int i = 0; i < n; ++i)
                if (hit[i] != 1) { printf("FAIL job %d index %d ran %d times\n", it, i, hit[i]); return 1; }
            if (it % 400 == 0) std::this_thread::sleep_for(std::chrono::milliseconds(3));   // workers sleep
        }
        printf("workers %d ok\n", workers);
    }
    return 0;
}
"""


def _build(tmp_path, extra):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    src = tmp_path / "pool_stress.cpp"
    src.write_text(STRESS)
    exe = tmp_path / "pool_stress"
    r = subprocess.run([cxx, "-std=c++17", "-pthread", "-I", CSRC, "-DNR_POOL_SPIN_US=300", *extra,
                        str(src), "-o", str(exe)], capture_output=True, text=True)
    return exe, r


def test_pool_runs_every_index_once(tmp_path):
    exe, r = _build(tmp_path, ["-O2"])
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe), "2000"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.count(" ok") == 3


def test_pool_under_thread_sanitizer(tmp_path):
    exe, r = _build(tmp_path, ["-O1", "-g", "-fsanitize=thread"])
    if r.returncode != 0:
        pytest.skip("no ThreadSanitizer runtime: " + r.stderr.strip()[:200])
    out = subprocess.run([str(exe), "150"], capture_output=True, text=True, timeout=600)
    if "FATAL: ThreadSanitizer" in out.stderr:
        pytest.skip("ThreadSanitizer cannot run here: " + out.stderr.strip()[:200])
    assert "WARNING: ThreadSanitizer" not in out.stderr, out.stderr[:4000]
    assert out.returncode == 0, out.stdout + out.stderr[:2000]
    assert out.stdout.count(" ok") == 3
