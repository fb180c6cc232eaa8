// Host side of unresize: the FP64 context of one axis, as zimg builds it
// (src/zimg/unresize/bilinear.cpp:20-170 over common/matrix.cpp's RowMatrix
// rules), and the pass order (unresize.cpp:14-19).
#include "unresize.h"

#include <algorithm>
#include <cfloat>
#include <cmath>

namespace zg {

namespace {

// Up to two (column, weight) entries of A's row i: the bilinear weights of
// upsampled sample i over the original samples, edges mirrored to the
// nearest sample (bilinear.cpp:60-104). A zero weight is no entry: zimg's
// matrix does not grow a row for a write of the value it already holds.
int bilinear_entries(unsigned in, unsigned out, double shift, unsigned i, unsigned col[2], double w[2])
{
	const double leftmost = 0.5 + shift, rightmost = in - 0.5 + shift;
	const unsigned lidx = static_cast<unsigned>(std::clamp(std::floor(leftmost), 0.0, in - 1.0));
	const unsigned ridx = static_cast<unsigned>(std::clamp(std::floor(rightmost), 0.0, in - 1.0));
	const double pos = (i + 0.5) * in / out;
	if (pos <= leftmost) {
		col[0] = lidx;
		w[0] = 1.0;
		return 1;
	}
	if (pos >= rightmost) {
		col[0] = ridx;
		w[0] = 1.0;
		return 1;
	}
	const unsigned left = static_cast<unsigned>(std::floor(pos - leftmost));
	const double dist = pos - left - leftmost;
	int n = 0;
	if (1.0 - dist != 0.0) {
		col[n] = left;
		w[n++] = 1.0 - dist;
	}
	if (dist != 0.0) {
		col[n] = left + 1;
		w[n++] = dist;
	}
	return n;
}

} // namespace

bool build_unresize_context(unsigned orig, unsigned up, double shift, UnresizeContext *out)
{
	if (orig > up)
		return false;
	const unsigned N = orig, M = up;
	const double s = -shift * N / M;  // output shift on the input grid
	std::vector<unsigned> col(2 * static_cast<size_t>(M));
	std::vector<double> wt(2 * static_cast<size_t>(M));
	std::vector<int> cnt(M);
	// A' row r spans A's rows [lo, hi): the first and last with an entry in column r
	std::vector<size_t> lo(N, 0), hi(N, 0);
	for (unsigned i = 0; i < M; ++i) {
		cnt[i] = bilinear_entries(N, M, s, i, &col[2 * i], &wt[2 * i]);
		for (int e = 0; e < cnt[i]; ++e) {
			const unsigned r = col[2 * i + e];
			if (hi[r] == 0)
				lo[r] = i;
			hi[r] = i + 1;
		}
	}
	auto a = [&](size_t i, unsigned c) {
		for (int e = 0; e < cnt[i]; ++e)
			if (col[2 * i + e] == c)
				return wt[2 * i + e];
		return 0.0;
	};
	// the band of A'A, each term summed over A' row r's run in order
	std::vector<double> pl(N, 0.0), pd(N, 0.0), pu(N, 0.0);
	unsigned row_size = 0;
	for (unsigned r = 0; r < N; ++r) {
		double acc[3] = { 0.0, 0.0, 0.0 };
		for (int t = 0; t < 3; ++t) {
			const long c = static_cast<long>(r) - 1 + t;
			if (c < 0 || c >= static_cast<long>(N))
				continue;
			double sum = 0.0;
			for (size_t k = lo[r]; k < hi[r]; ++k) {
				const double prod = a(k, r) * a(k, static_cast<unsigned>(c));
				sum = sum + prod;
			}
			acc[t] = sum;
		}
		pl[r] = acc[0];
		pd[r] = acc[1];
		pu[r] = acc[2];
		row_size = std::max(row_size, static_cast<unsigned>(hi[r] - lo[r]));
	}
	// tridiagonal LU with DBL_EPSILON guards on the divisors
	std::vector<double> c(N, 0.0), l(N, 0.0), u(N, 0.0);
	const double eps = DBL_EPSILON;
	if (N == 1) {
		l[0] = pd[0];
	} else {
		l[0] = pd[0];
		u[0] = pu[0] / (pd[0] + eps);
		for (unsigned i = 1; i + 1 < N; ++i) {
			c[i] = pl[i];
			l[i] = pd[i] - c[i] * u[i - 1];
			u[i] = pu[i] / (l[i] + eps);
		}
		c[N - 1] = pl[N - 1];
		l[N - 1] = pd[N - 1] - c[N - 1] * u[N - 2];
	}
	UnresizeContext &x = *out;
	x.up = M;
	x.orig = N;
	x.row_size = row_size;
	x.coef.assign(static_cast<size_t>(N) * std::max(row_size, 1u), 0.0f);
	x.offset.assign(N, 0);
	x.lu_c.resize(N);
	x.lu_l.resize(N);
	x.lu_u.resize(N);
	for (unsigned r = 0; r < N; ++r) {
		// the run starts early enough that row_size samples fit in the line
		const size_t left = hi[r] ? std::min(lo[r], static_cast<size_t>(M - row_size)) : 0;
		for (size_t k = left; hi[r] && k < hi[r]; ++k)
			x.coef[static_cast<size_t>(r) * row_size + (k - left)] = static_cast<float>(a(k, r));
		x.offset[r] = static_cast<unsigned>(left);
		x.lu_c[r] = static_cast<float>(c[r]);
		x.lu_l[r] = static_cast<float>(1.0 / (l[r] + eps));
		x.lu_u[r] = static_cast<float>(u[r]);
	}
	return true;
}

bool unresize_h_first(double xscale, double yscale)
{
	const double h = std::max(xscale, 1.0) * 2.0 + xscale * std::max(yscale, 1.0);
	const double v = std::max(yscale, 1.0) + yscale * std::max(xscale, 1.0) * 2.0;
	return h < v;
}

} // namespace zg
