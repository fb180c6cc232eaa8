// Guided chunks of a persistent launch's work units (work_chunks.h).
#include "work_chunks.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>

namespace zg {

std::vector<int> chain_mixed_chunks(const std::vector<int> &item_begin, const std::vector<int> &items,
                                    const std::vector<double> &cost, const std::vector<int> &strip_units, int grid,
                                    int min_units)
{
	const size_t n = items.size();
	if (n == 0 || item_begin.size() != n || cost.size() != n || strip_units.size() != n || grid < 1)
		return {};
	const int units = item_begin[n - 1] + items[n - 1];
	double left = 0;
	for (size_t e = 0; e < n; ++e)
		left += cost[e] * items[e];
	std::vector<int> bounds{ item_begin[0] };
	size_t e = 0;  // job of unit u
	int u = item_begin[0];
	while (u < units) {
		const double want = left / (2.0 * grid);
		double got = 0;
		int v = u;
		size_t f = e;
		while (v < units && (got < want || v - u < min_units)) {
			while (f + 1 < n && v >= item_begin[f] + items[f])
				++f;
			const int room = item_begin[f] + items[f] - v;
			const double c = std::max(cost[f], 1e-30);
			int k = static_cast<int>(std::ceil((want - got) / c));
			k = std::max(k, min_units - (v - u));
			k = std::max(1, std::min(k, room));
			v += k;
			got += k * cost[f];
		}
		// inside a job with strips: end on the nearest strip boundary past u
		// where that changes the chunk by at most a quarter
		if (v < units && strip_units[f] > 0 && v > item_begin[f]) {
			const int su = strip_units[f], off = v - item_begin[f];
			int w = item_begin[f] + (off + su / 2) / su * su;
			if (w <= u)
				w = item_begin[f] + (off / su + 1) * su;
			w = std::min(w, item_begin[f] + items[f]);
			if (4 * std::abs(w - v) <= v - u) {
				got += (w - v) * cost[f];  // units moved in (or out)
				v = w;
			}
		}
		bounds.push_back(v);
		left -= got;
		u = v;
		e = f;
	}
	return bounds;
}

} // namespace zg
