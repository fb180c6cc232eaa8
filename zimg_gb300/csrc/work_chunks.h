// Guided chunks of a persistent launch's work units, planned on the host
// (the device side is work_chunks.cuh). Plain C++: no CUDA types.
#pragma once

#include <vector>

namespace zg {

// Guided chunk bounds: the units of jobs with item_begin[e] ..
// item_begin[e] + items[e] - 1 (in order, contiguous) at an estimated cost
// per unit cost[e]; each chunk takes 1 / (2 grid) of the cost still left, but
// at least min_units units (or the rest), and a chunk that ends inside a job
// with strip_units[e] > 0 units per strip ends on the nearest strip boundary
// instead where that changes it by at most a quarter (a chunk that splits a
// strip makes its tail a second item, which starts its pipeline again).
// Returns the bounds (chunk m: [bounds[m], bounds[m + 1])), strictly
// increasing, from the first job's first unit to the last job's end; empty
// for inconsistent arguments.
std::vector<int> chain_mixed_chunks(const std::vector<int> &item_begin, const std::vector<int> &items,
                                    const std::vector<double> &cost, const std::vector<int> &strip_units, int grid,
                                    int min_units);

} // namespace zg
