"""The heap-order simulation's queue (csrc/tie_heap.h) pops, ties included, in the order of
std::priority_queue<QueueItem> (the reference propagation's queue, reliability_propagation.cpp:
44-53): a C++ differential test over random pushes and pops with heavy ties, double and float
keys, built with the host compiler."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "traditional-dic_gb300", "csrc")

_PROGRAM = r"""
#include "tie_heap.h"
#include <cstdio>
#include <queue>
#include <random>
struct Item {
    double k;
    int n;
    bool operator<(const Item& o) const { return k > o.k; }
};
int main() {
    std::mt19937_64 rng(7);
    long long ops = 0, bad = 0;
    for (int trial = 0; trial < 1500; ++trial) {
        std::priority_queue<Item> ref;
        tdic::TieHeap<double> hd;
        tdic::TieHeap<float> hf;
        const int distinct = 1 + (int)(rng() % (trial % 7 == 0 ? 3 : 50));
        const int steps = 50 + (int)(rng() % 3000);
        int id = 0;
        auto check = [&]() { if (ref.top().n != hd.top() || ref.top().n != hf.top()) ++bad; };
        for (int s = 0; s < steps; ++s, ++ops) {
            if (ref.empty() || rng() % 100 < 55) {
                const double k = (double)(float)((rng() % distinct) * 0.125 + ((trial & 1) ? 0.0 : 1e-3));
                ref.push(Item{k, id}); hd.push(k, id); hf.push((float)k, id); ++id;
            } else {
                check(); ref.pop(); hd.pop(); hf.pop();
            }
        }
        while (!ref.empty()) { check(); ref.pop(); hd.pop(); hf.pop(); ++ops; }
        if (!hd.empty() || !hf.empty()) ++bad;
    }
    std::printf("%lld %lld\n", ops, bad);
    return bad != 0;
}
"""


def test_tie_heap_pops_like_std_priority_queue(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "tie_heap_test.cpp"
    src.write_text(_PROGRAM)
    exe = tmp_path / "tie_heap_test"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    ops, bad = map(int, r.stdout.split())
    assert r.returncode == 0 and bad == 0 and ops > 1_000_000
