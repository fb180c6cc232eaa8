"""Guided work chunks (zimg_gb300/csrc/work_chunks.cpp), host logic on CPU.

A persistent launch's CTAs take chunks of its work units from a counter; the
host cuts the units into chunks of decreasing estimated cost (1 / (2 grid) of
the cost left, at least min_units, ending on strip boundaries where that
moves the end by at most a quarter). These tests compile the planner with g++
and check its invariants on job mixes like the batches that use it.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "zimg_gb300", "csrc")

DRIVER = r"""
#include "work_chunks.h"
#include <cstdio>
#include <vector>

// one scenario per line of stdin: grid min_units n, then n lines "begin items cost strip_units"
int main()
{
	int grid, min_units, n;
	while (std::scanf("%d %d %d", &grid, &min_units, &n) == 3) {
		std::vector<int> ib(n), it(n), su(n);
		std::vector<double> c(n);
		for (int e = 0; e < n; ++e)
			std::scanf("%d %d %lf %d", &ib[e], &it[e], &c[e], &su[e]);
		const std::vector<int> b = zg::chain_mixed_chunks(ib, it, c, su, grid, min_units);
		std::printf("[");
		for (size_t i = 0; i < b.size(); ++i)
			std::printf(i ? ",%d" : "%d", b[i]);
		std::printf("]\n");
	}
	return 0;
}
"""


@pytest.fixture(scope="module")
def planner(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("chunks")
    drv = d / "driver.cpp"
    drv.write_text(DRIVER)
    exe = d / "chunks"
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", CSRC, str(drv), os.path.join(CSRC, "work_chunks.cpp"),
                    "-o", str(exe)], check=True, capture_output=True)

    def run(grid, min_units, jobs):
        text = f"{grid} {min_units} {len(jobs)}\n" + "".join(f"{b} {n} {c} {s}\n" for b, n, c, s in jobs)
        out = subprocess.run([str(exe)], input=text, capture_output=True, text=True, check=True).stdout
        return json.loads(out.strip())
    return run


def contiguous(jobs_spec, start=0):
    """(items, cost, strip_units) triples -> (begin, items, cost, strip_units) with contiguous units."""
    out, u = [], start
    for n, c, s in jobs_spec:
        out.append((u, n, c, s))
        u += n
    return out


def job_of(jobs, v):
    for b, n, c, s in jobs:
        if b <= v < b + n:
            return b, n, c, s
    return jobs[-1]


def chunk_cost(jobs, a, b):
    total = 0.0
    for jb, n, c, _ in jobs:
        lo, hi = max(a, jb), min(b, jb + n)
        if hi > lo:
            total += (hi - lo) * c
    return total


def check(jobs, bounds, grid, min_units):
    assert bounds[0] == jobs[0][0] and bounds[-1] == jobs[-1][0] + jobs[-1][1]
    assert all(b > a for a, b in zip(bounds, bounds[1:])), "bounds strictly increasing"
    sizes = [b - a for a, b in zip(bounds, bounds[1:])]
    # at least min_units (a strip snap may take off a quarter), except the last chunk
    assert all(s >= (3 * min_units) // 4 for s in sizes[:-1]), min(sizes[:-1])
    # guided: the first chunk takes about 1 / (2 grid) of the whole cost
    total = chunk_cost(jobs, bounds[0], bounds[-1])
    first = chunk_cost(jobs, bounds[0], bounds[1])
    assert first <= 1.3 * total / (2 * grid) + max(c for _, _, c, _ in jobs) * min_units
    # a chunk end inside a strip is further than a quarter of its chunk from the nearest boundary
    for a, v in zip(bounds, bounds[1:-1]):
        b, n, c, s = job_of(jobs, v)
        if s > 0 and v > b and (v - b) % s:
            off = v - b
            w = b + (off + s // 2) // s * s
            if w <= a:
                w = b + (off // s + 1) * s
            w = min(w, b + n)
            assert 4 * abs(w - v) > v - a, (a, v, w)
    return sizes


def test_yuv_like_mix(planner):
    # 2160p downscales (68 units per strip), 1.5x / 2.25x upscales, then identity copies (no strips)
    spec = []
    for _ in range(19):
        spec += [(1020, 30000.0, 68), (510, 30000.0, 34), (510, 30000.0, 34)]
    for _ in range(30):
        spec += [(360, 12000.0, 68), (180, 12000.0, 34), (180, 12000.0, 34)]
    spec += [(68, 9000.0, 0)] * 45
    jobs = contiguous(spec)
    bounds = planner(304, 12, jobs)
    sizes = check(jobs, bounds, 304, 12)
    assert len(sizes) > 304  # more chunks than CTAs: the tail is fine-grained
    assert sizes[-1] <= 68 and sizes[0] > sizes[-1]


def test_single_job_many_strips(planner):
    # one CUDA-core streaming job of 384 planes x 10 strips x 90 steps, strip = 90 units
    jobs = contiguous([(345600, 1.0, 90)])
    bounds = planner(760, 8, jobs)
    sizes = check(jobs, bounds, 760, 8)
    # early chunks are whole strips: they end on strip boundaries
    assert all(b % 90 == 0 for b in bounds[1:200])
    assert sizes[0] >= 180 and min(sizes) >= 6


def test_offset_start_and_tiny(planner):
    jobs = contiguous([(50, 2.0, 10), (7, 1.0, 0)], start=1000)
    bounds = planner(4, 3, jobs)
    check(jobs, bounds, 4, 3)
    assert planner(304, 12, contiguous([(5, 1.0, 0)])) == [0, 5]


def test_inconsistent_arguments(planner):
    assert planner(0, 12, contiguous([(10, 1.0, 0)])) == []
