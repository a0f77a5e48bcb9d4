"""Host thread helpers of the library (csrc/host_sparse.hpp): parallel_for
and run_pair, with and without the NSS_HOST_THREADS cap.

The header is compiled here with the host C++ compiler into a small test
program; no GPU and no CUDA toolkit are involved.  The program
prints one line per check; the test reads them back.
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER_DIR = ROOT / "nssdmrg_gb300" / "csrc"

PROGRAM = r"""
#include "host_sparse.hpp"
#include <cstdio>
#include <stdexcept>
#include <thread>

using namespace nss;

int main() {
    // every index exactly once, on more than one thread when allowed
    {
        const int n = 5000;
        std::vector<std::atomic<int>> hits(n);
        for (auto &h : hits) h = 0;
        std::mutex mu;
        std::set<std::thread::id> ids;
        parallel_for(n, [&](int i) {
            hits[i]++;
            std::lock_guard<std::mutex> lk(mu);
            ids.insert(std::this_thread::get_id());
        });
        int bad = 0;
        for (auto &h : hits) bad += h.load() != 1;
        std::printf("cover %d %zu\n", bad, ids.size());
    }
    // serial: parallel=false, n < 2
    {
        std::vector<int> order;
        parallel_for(4, [&](int i) { order.push_back(i); }, false);
        parallel_for(1, [&](int i) { order.push_back(10 + i); });
        parallel_for(0, [&](int) { order.push_back(-1); });
        std::printf("serial");
        for (int x : order) std::printf(" %d", x);
        std::printf("\n");
    }
    // an exception in one index reaches the caller after the others stop
    {
        std::atomic<int> ran{0};
        try {
            parallel_for(2000, [&](int i) {
                ran++;
                if (i == 700) throw std::runtime_error("index 700");
            });
            std::printf("throw none\n");
        } catch (const std::exception &e) {
            std::printf("throw %s %d\n", e.what(), ran.load() <= 2000 ? 1 : 0);
        }
    }
    // run_pair: both run; f0's exception first
    {
        int a = 0, b = 0;
        run_pair([&] { a = 1; }, [&] { b = 2; });
        std::string which = "none";
        try {
            run_pair([&] { throw std::runtime_error("f0"); }, [&] { throw std::runtime_error("f1"); });
        } catch (const std::exception &e) {
            which = e.what();
        }
        std::printf("pair %d %d %s\n", a, b, which.c_str());
    }
    std::printf("cap %d\n", host_threads_cap() >= (1 << 20) ? 0 : host_threads_cap());
    return 0;
}
"""


@pytest.fixture(scope="module")
def helper_exe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("host_parallel")
    src, exe = d / "check.cpp", d / "check"
    src.write_text("#include <mutex>\n#include <set>\n" + PROGRAM)
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-pthread", f"-I{HEADER_DIR}", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def _run(exe, threads=None):
    env = dict(os.environ)
    env.pop("NSS_HOST_THREADS", None)
    if threads is not None:
        env["NSS_HOST_THREADS"] = str(threads)
    out = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=60)
    assert out.returncode == 0, out.stderr
    return {ln.split()[0]: ln.split()[1:] for ln in out.stdout.splitlines()}


def test_parallel_for_covers_every_index_once(helper_exe):
    res = _run(helper_exe)
    bad, nthreads = int(res["cover"][0]), int(res["cover"][1])
    assert bad == 0
    if (os.cpu_count() or 1) > 1:
        assert nthreads > 1
    assert res["serial"] == ["0", "1", "2", "3", "10"]
    assert res["throw"][:2] == ["index", "700"]
    assert res["pair"] == ["1", "2", "f0"]
    assert res["cap"] == ["0"]


def test_host_thread_cap_of_one_runs_on_the_caller(helper_exe):
    res = _run(helper_exe, threads=1)
    assert res["cover"] == ["0", "1"]          # every index, one thread
    assert res["serial"] == ["0", "1", "2", "3", "10"]
    assert res["throw"][:2] == ["index", "700"]
    assert res["pair"] == ["1", "2", "f0"]
    assert res["cap"] == ["1"]
