// Host planning of a colorspace conversion: zimg's path search between
// colorspaces (src/zimg/colorspace/colorspace_graph.cpp:117-245), the 3x3
// matrices of each step in double (colorspace_param.cpp, matrix3.cpp; the
// colorimetry is ITU-T H.273 / BT.709 / BT.2020 / BT.2100 constants, RGB to
// XYZ after Lindbloom, Bradford white-point adaptation), and the float
// parameters of each per-pixel operation (operation.cpp,
// operation_impl.cpp:263-385).
#include "colorspace_plan.h"

#include <array>
#include <deque>
#include <unordered_map>
#include <vector>

#include "capi_common.h"
#include "colorspace_tf.cuh"

namespace zg {
namespace csp {

namespace {

struct V3 {
	double v[3];
	double operator[](int i) const { return v[i]; }
};

struct M3 {
	double a[3][3];

	static M3 identity() { return { { { 1, 0, 0 }, { 0, 1, 0 }, { 0, 0, 1 } } }; }

	M3 operator*(const M3 &b) const
	{
		M3 r{};
		for (int i = 0; i < 3; ++i)
			for (int j = 0; j < 3; ++j) {
				double acc = 0;
				for (int k = 0; k < 3; ++k)
					acc += a[i][k] * b.a[k][j];
				r.a[i][j] = acc;
			}
		return r;
	}

	V3 operator*(const V3 &x) const
	{
		V3 r{};
		for (int i = 0; i < 3; ++i) {
			double acc = 0;
			for (int k = 0; k < 3; ++k)
				acc += a[i][k] * x.v[k];
			r.v[i] = acc;
		}
		return r;
	}
};

double minor2(double p, double q, double r, double s)
{
	return p * s - q * r;
}

// Cofactor inverse, the order of zimg's matrix3.cpp:63-99 (the rounding of
// the FP64 entries is part of the result).
M3 inverse(const M3 &m)
{
	const auto &a = m.a;
	double det = 0;
	det += a[0][0] * minor2(a[1][1], a[1][2], a[2][1], a[2][2]);
	det -= a[0][1] * minor2(a[1][0], a[1][2], a[2][0], a[2][2]);
	det += a[0][2] * minor2(a[1][0], a[1][1], a[2][0], a[2][1]);
	M3 r;
	r.a[0][0] = minor2(a[1][1], a[1][2], a[2][1], a[2][2]) / det;
	r.a[0][1] = minor2(a[0][2], a[0][1], a[2][2], a[2][1]) / det;
	r.a[0][2] = minor2(a[0][1], a[0][2], a[1][1], a[1][2]) / det;
	r.a[1][0] = minor2(a[1][2], a[1][0], a[2][2], a[2][0]) / det;
	r.a[1][1] = minor2(a[0][0], a[0][2], a[2][0], a[2][2]) / det;
	r.a[1][2] = minor2(a[0][2], a[0][0], a[1][2], a[1][0]) / det;
	r.a[2][0] = minor2(a[1][0], a[1][1], a[2][0], a[2][1]) / det;
	r.a[2][1] = minor2(a[0][1], a[0][0], a[2][1], a[2][0]) / det;
	r.a[2][2] = minor2(a[0][0], a[0][1], a[1][0], a[1][1]) / det;
	return r;
}

V3 cross(const V3 &x, const V3 &y)
{
	return { { x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0] } };
}

double dot(const V3 &x, const V3 &y)
{
	return x[0] * y[0] + x[1] * y[1] + x[2] * y[2];
}

// chromaticity (x, y) -> XYZ with Y = 1
V3 xyz_of(double x, double y)
{
	return { { x / y, 1.0, (1.0 - x - y) / y } };
}

// White points: illuminant C, E, the DCI white, D65.
V3 white_of(int p)
{
	switch (p) {
	case P_470M:
	case P_FILM: return xyz_of(0.31, 0.316);
	case P_XYZ: return xyz_of(1.0 / 3.0, 1.0 / 3.0);
	case P_DCI_P3: return xyz_of(0.314, 0.351);
	default: return xyz_of(0.3127, 0.3290);
	}
}

// R, G, B chromaticities of each primaries set (H.273 table 2).
std::array<std::array<double, 2>, 3> chroma_of(int p)
{
	switch (p) {
	case P_470M: return { { { 0.670, 0.330 }, { 0.210, 0.710 }, { 0.140, 0.080 } } };
	case P_470BG: return { { { 0.640, 0.330 }, { 0.290, 0.600 }, { 0.150, 0.060 } } };
	case P_SMPTE_C: return { { { 0.630, 0.340 }, { 0.310, 0.595 }, { 0.155, 0.070 } } };
	case P_FILM: return { { { 0.681, 0.319 }, { 0.243, 0.692 }, { 0.145, 0.049 } } };
	case P_2020: return { { { 0.708, 0.292 }, { 0.170, 0.797 }, { 0.131, 0.046 } } };
	case P_DCI_P3:
	case P_DCI_P3_D65: return { { { 0.680, 0.320 }, { 0.265, 0.690 }, { 0.150, 0.060 } } };
	case P_EBU_3213_E: return { { { 0.630, 0.340 }, { 0.295, 0.605 }, { 0.155, 0.077 } } };
	default: return { { { 0.640, 0.330 }, { 0.300, 0.600 }, { 0.150, 0.060 } } };
	}
}

// Y'CbCr from R'G'B' for luma weights kr, kb
M3 yuv_from_kr_kb(double kr, double kb)
{
	const double kg = 1.0 - kr - kb;
	const double us = 1.0 / (2.0 - 2.0 * kb), vs = 1.0 / (2.0 - 2.0 * kr);
	return { { { kr, kg, kb }, { -kr * us, -kg * us, (1.0 - kb) * us }, { (1.0 - kr) * vs, -kg * vs, -kb * vs } } };
}

M3 rgb_to_yuv(int m)
{
	switch (m) {
	case M_YCGCO: return { { { 0.25, 0.5, 0.25 }, { -0.25, 0.5, -0.25 }, { 0.5, 0, -0.5 } } };
	case M_LMS:
		return { { { 1688.0 / 4096.0, 2146.0 / 4096.0, 262.0 / 4096.0 },
		           { 683.0 / 4096.0, 2951.0 / 4096.0, 462.0 / 4096.0 },
		           { 99.0 / 4096.0, 309.0 / 4096.0, 3688.0 / 4096.0 } } };
	case M_FCC: return yuv_from_kr_kb(0.3, 0.11);
	case M_240M: return yuv_from_kr_kb(0.212, 0.087);
	case M_601: return yuv_from_kr_kb(0.299, 0.114);
	case M_709: return yuv_from_kr_kb(0.2126, 0.0722);
	case M_2020_NCL:
	case M_2020_CL: return yuv_from_kr_kb(0.2627, 0.0593);
	default: throw Error(kErrLogic, "unrecognized matrix coefficients");
	}
}

// Luma weights from the primaries' chromaticities and white (H.273 E-22..E-27).
M3 rgb_to_yuv_from_primaries(int p)
{
	if (p == P_709)
		return rgb_to_yuv(M_709);
	if (p == P_2020)
		return rgb_to_yuv(M_2020_NCL);
	const auto c = chroma_of(p);
	const V3 r = xyz_of(c[0][0], c[0][1]), g = xyz_of(c[1][0], c[1][1]), b = xyz_of(c[2][0], c[2][1]);
	const V3 w = white_of(p);
	const V3 xs{ { r[0], g[0], b[0] } }, ys{ { r[1], g[1], b[1] } }, zs{ { r[2], g[2], b[2] } };
	const double den = dot(xs, cross(ys, zs));
	return yuv_from_kr_kb(dot(w, cross(g, b)) / den, dot(w, cross(r, g)) / den);
}

M3 lms_to_ictcp(int t)
{
	if (t == T_B67)
		return { { { 0.5, 0.5, 0.0 }, { 3625.0 / 4096.0, -7465.0 / 4096.0, 3840.0 / 4096.0 },
		           { 9500.0 / 4096.0, -9212.0 / 4096.0, -288.0 / 4096.0 } } };
	return { { { 0.5, 0.5, 0.0 }, { 6610.0 / 4096.0, -13613.0 / 4096.0, 7003.0 / 4096.0 },
	           { 17933.0 / 4096.0, -17390.0 / 4096.0, -543.0 / 4096.0 } } };
}

M3 rgb_to_xyz(int p)
{
	if (p == P_XYZ)
		return M3::identity();
	const auto c = chroma_of(p);
	M3 cols{};  // columns: the primaries' XYZ
	for (int k = 0; k < 3; ++k) {
		const V3 v = xyz_of(c[k][0], c[k][1]);
		for (int r = 0; r < 3; ++r)
			cols.a[r][k] = v[r];
	}
	const V3 s = inverse(cols) * white_of(p);
	M3 m{};
	for (int r = 0; r < 3; ++r)
		for (int k = 0; k < 3; ++k)
			m.a[r][k] = cols.a[r][k] * s[k];
	return m;
}

M3 xyz_to_rgb(int p)
{
	return p == P_XYZ ? M3::identity() : inverse(rgb_to_xyz(p));
}

M3 bradford(int in, int out)
{
	const M3 b = { { { 0.8951, 0.2664, -0.1614 }, { -0.7502, 1.7135, 0.0367 }, { 0.0389, -0.0685, 1.0296 } } };
	const V3 wi = white_of(in), wo = white_of(out);
	if (wi[0] == wo[0] && wi[1] == wo[1] && wi[2] == wo[2])
		return M3::identity();
	const V3 ci = b * wi, co = b * wo;
	M3 d{};
	for (int k = 0; k < 3; ++k)
		d.a[k][k] = co[k] / ci[k];
	return inverse(b) * d * b;
}

// select_transfer_function (gamma.cpp:346-411): function ids and scales
struct Transfer_ {
	int to_linear, to_gamma;
	float linear_scale = 1.0f, gamma_scale = 1.0f;
};

Transfer_ transfer_of(int t, double peak, bool scene)
{
	Transfer_ f{ -1, -1 };
	switch (t) {
	case T_LOG100: f.to_linear = TF_LOG100_INV; f.to_gamma = TF_LOG100; break;
	case T_LOG316: f.to_linear = TF_LOG316_INV; f.to_gamma = TF_LOG316; break;
	case T_709:
		f.to_linear = scene ? TF_709_INV_OETF : TF_1886;
		f.to_gamma = scene ? TF_709_OETF : TF_1886_INV;
		break;
	case T_470M: f.to_linear = TF_470M; f.to_gamma = TF_470M_INV; break;
	case T_470BG: f.to_linear = TF_470BG; f.to_gamma = TF_470BG_INV; break;
	case T_240M:
		f.to_linear = scene ? TF_240M_INV_OETF : TF_1886;
		f.to_gamma = scene ? TF_240M_OETF : TF_1886_INV;
		break;
	case T_1361:
		f.to_linear = scene ? TF_1361_INV_OETF : TF_1361_EOTF;
		f.to_gamma = scene ? TF_1361_OETF : TF_1361_INV_EOTF;
		break;
	case T_XVYCC:
		f.to_linear = scene ? TF_XVYCC_INV_OETF : TF_XVYCC_EOTF;
		f.to_gamma = scene ? TF_XVYCC_OETF : TF_XVYCC_INV_EOTF;
		break;
	case T_SRGB: f.to_linear = TF_SRGB; f.to_gamma = TF_SRGB_INV; break;
	case T_2084:
		f.to_linear = scene ? TF_PQ_INV_OETF : TF_PQ_EOTF;
		f.to_gamma = scene ? TF_PQ_OETF : TF_PQ_INV_EOTF;
		f.linear_scale = static_cast<float>(10000.0f / peak);
		f.gamma_scale = static_cast<float>(peak / 10000.0f);
		break;
	case T_428: f.to_linear = TF_428; f.to_gamma = TF_428_INV; break;
	case T_B67:
		f.to_linear = scene ? TF_HLG_INV_OETF : TF_HLG_EOTF;
		f.to_gamma = scene ? TF_HLG_OETF : TF_HLG_INV_EOTF;
		f.linear_scale = scene ? 12.0f : static_cast<float>(1000.0 / peak);
		f.gamma_scale = scene ? 1.0f / 12.0f : static_cast<float>(peak / 1000.0);
		break;
	default: throw Error(kErrLogic, "invalid transfer characteristics");
	}
	return f;
}

// validity of a colorspace (is_valid_csp, colorspace_graph.cpp:70-101)
bool valid(const Space &c)
{
	if (c.m == M_2020_CL && c.t != T_709)
		return false;
	if ((c.m == M_CHROM_NCL || c.m == M_CHROM_CL) && c.p == P_UNSPEC)
		return false;
	if (c.m == M_ICTCP && !((c.t == T_2084 || c.t == T_B67) && c.p == P_2020))
		return false;
	if (c.m == M_LMS && !((c.t == T_LINEAR || c.t == T_2084 || c.t == T_B67) && c.p == P_2020))
		return false;
	return true;
}

enum Step : int { S_NCL_TO_RGB, S_NCL_TO_YUV, S_ICTCP_TO_LMS, S_LMS_TO_ICTCP, S_TO_LINEAR, S_TO_GAMMA, S_CL_TO_RGB,
                  S_CL_TO_YUV, S_GAMUT };

struct Edge {
	Space to;
	int step;
};

// The neighbours of a colorspace in zimg's order (colorspace_graph.cpp:117-193).
std::vector<Edge> neighbours(const Space &c)
{
	std::vector<Edge> e;
	auto add = [&](int m, int t, int p, int s) { e.push_back({ Space{ m, t, p }, s }); };
	if (c.m == M_RGB) {
		for (int m = 0; m < M_COUNT; ++m) {
			const bool special = m == M_UNSPEC || m == M_RGB || m == M_2020_CL || m == M_CHROM_NCL || m == M_CHROM_CL ||
			                     m == M_LMS || m == M_ICTCP;
			if (!special)
				add(m, c.t, c.p, S_NCL_TO_YUV);
		}
		if (c.p != P_UNSPEC)
			add(M_CHROM_NCL, c.t, c.p, S_NCL_TO_YUV);
		if (c.t == T_LINEAR) {
			for (int t = 0; t < T_COUNT; ++t) {
				if (t == c.t || t == T_UNSPEC)
					continue;
				add(c.m, t, c.p, S_TO_GAMMA);
				if (c.p != P_UNSPEC)
					add(M_CHROM_CL, t, c.p, S_CL_TO_YUV);
			}
			if (c.p != P_UNSPEC)
				for (int p = 0; p < P_COUNT; ++p)
					if (p != c.p && p != P_UNSPEC)
						add(c.m, c.t, p, S_GAMUT);
			add(M_2020_CL, T_709, c.p, S_CL_TO_YUV);
			if (c.p == P_2020)
				add(M_LMS, c.t, c.p, S_NCL_TO_YUV);
		} else if (c.t != T_UNSPEC) {
			add(c.m, T_LINEAR, c.p, S_TO_LINEAR);
		}
	} else if (c.m == M_2020_CL || c.m == M_CHROM_CL) {
		add(M_RGB, T_LINEAR, c.p, S_CL_TO_RGB);
	} else if (c.m == M_LMS) {
		if (c.t == T_2084 || c.t == T_B67) {
			add(M_ICTCP, c.t, c.p, S_LMS_TO_ICTCP);
			add(c.m, T_LINEAR, c.p, S_TO_LINEAR);
		}
		if (c.t == T_LINEAR) {
			add(M_RGB, c.t, c.p, S_NCL_TO_RGB);
			add(c.m, T_2084, c.p, S_TO_GAMMA);
			add(c.m, T_B67, c.p, S_TO_GAMMA);
		}
	} else if (c.m == M_ICTCP) {
		if (c.t == T_2084 || c.t == T_B67)
			add(M_LMS, c.t, c.p, S_ICTCP_TO_LMS);
	} else if (c.m != M_UNSPEC) {
		add(M_RGB, c.t, c.p, S_NCL_TO_RGB);
	}
	return e;
}

int key_of(const Space &c)
{
	return (c.m * T_COUNT + c.t) * P_COUNT + c.p;
}

Op matrix_op(const M3 &m)
{
	Op o{};
	o.kind = OP_MATRIX;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			o.m[i][j] = static_cast<float>(m.a[i][j]);
	return o;
}

// chroma scales of the constant-luminance operations, evaluated on the host
// as zimg evaluates them (operation_impl.cpp:180-186, 236-242)
void cl_scales(Op &o, int to_gamma)
{
	o.nb = apply_tf(to_gamma, 1.0f - o.kb);
	o.pb = 1.0f - apply_tf(to_gamma, o.kb);
	o.nr = apply_tf(to_gamma, 1.0f - o.kr);
	o.pr = 1.0f - apply_tf(to_gamma, o.kr);
}

Op make_op(int step, const Space &in, const Space &out, double peak, bool approx, bool scene, bool adapt)
{
	// display-referred HLG uses the luma-weighted OOTF (operation.cpp:16-19)
	auto hlg_display = [&](int p) { return p != P_UNSPEC && !approx && !scene; };
	Op o{};
	switch (step) {
	case S_NCL_TO_RGB:
		return matrix_op(inverse(in.m == M_CHROM_NCL ? rgb_to_yuv_from_primaries(in.p) : rgb_to_yuv(in.m)));
	case S_NCL_TO_YUV: return matrix_op(out.m == M_CHROM_NCL ? rgb_to_yuv_from_primaries(out.p) : rgb_to_yuv(out.m));
	case S_ICTCP_TO_LMS: return matrix_op(inverse(lms_to_ictcp(in.t)));
	case S_LMS_TO_ICTCP: return matrix_op(lms_to_ictcp(in.t));
	case S_TO_LINEAR:
		if (in.t == T_B67 && hlg_display(in.p)) {
			const M3 m = rgb_to_yuv_from_primaries(in.p);
			o.kind = OP_HLG_INV;
			o.kr = static_cast<float>(m.a[0][0]);
			o.kg = static_cast<float>(m.a[0][1]);
			o.kb = static_cast<float>(m.a[0][2]);
			o.scale = transfer_of(T_B67, peak, false).linear_scale;
		} else {
			const Transfer_ f = transfer_of(in.t, peak, scene);
			o.kind = OP_GAMMA;
			o.f = f.to_linear;
			o.pre = 1.0f;
			o.post = f.linear_scale;
		}
		return o;
	case S_TO_GAMMA:
		if (out.t == T_B67 && hlg_display(out.p)) {
			const M3 m = rgb_to_yuv_from_primaries(out.p);
			o.kind = OP_HLG;
			o.kr = static_cast<float>(m.a[0][0]);
			o.kg = static_cast<float>(m.a[0][1]);
			o.kb = static_cast<float>(m.a[0][2]);
			o.scale = transfer_of(T_B67, peak, false).gamma_scale;
		} else {
			const Transfer_ f = transfer_of(out.t, peak, scene);
			o.kind = OP_GAMMA;
			o.f = f.to_gamma;
			o.pre = f.gamma_scale;
			o.post = 1.0f;
		}
		return o;
	case S_GAMUT:
		return matrix_op(adapt ? xyz_to_rgb(out.p) * bradford(in.p, out.p) * rgb_to_xyz(in.p)
		                       : xyz_to_rgb(out.p) * rgb_to_xyz(in.p));
	case S_CL_TO_RGB:
	case S_CL_TO_YUV: {
		// constant luminance is always scene referred (operation_impl.cpp:360-384)
		const Space &cl = step == S_CL_TO_RGB ? in : out;
		const Transfer_ f = transfer_of(cl.t, peak, true);
		const M3 m = cl.m == M_CHROM_CL ? rgb_to_yuv_from_primaries(cl.p) : rgb_to_yuv(cl.m);
		o.kind = step == S_CL_TO_RGB ? OP_CL_TO_RGB : OP_CL_TO_YUV;
		o.f = step == S_CL_TO_RGB ? f.to_linear : f.to_gamma;
		o.g = f.to_gamma;
		o.kr = static_cast<float>(m.a[0][0]);
		o.kg = static_cast<float>(m.a[0][1]);
		o.kb = static_cast<float>(m.a[0][2]);
		o.scale = step == S_CL_TO_RGB ? f.linear_scale : f.gamma_scale;
		cl_scales(o, f.to_gamma);
		return o;
	}
	default: throw Error(kErrLogic, "unknown colorspace step");
	}
}

int lookup(int code, std::initializer_list<std::pair<int, int>> map, const char *what)
{
	if (code < 0 || code > 255)
		throw Error(kErrEnumOutOfRange, what);
	for (const auto &kv : map)
		if (kv.first == code)
			return kv.second;
	throw Error(kErrNoColorspaceConversion, what);
}

} // namespace

Space from_api(int matrix, int transfer, int primaries)
{
	// zimg.cpp:238-305
	Space s;
	s.m = lookup(matrix, { { 0, M_RGB }, { 1, M_709 }, { 2, M_UNSPEC }, { 4, M_FCC }, { 5, M_601 }, { 6, M_601 },
	                       { 7, M_240M }, { 8, M_YCGCO }, { 9, M_2020_NCL }, { 10, M_2020_CL }, { 12, M_CHROM_NCL },
	                       { 13, M_CHROM_CL }, { 14, M_ICTCP } },
	             "unrecognized matrix coefficients");
	s.t = lookup(transfer, { { 1, T_709 }, { 2, T_UNSPEC }, { 7, T_240M }, { 6, T_709 }, { 4, T_470M }, { 5, T_470BG },
	                         { 11, T_XVYCC }, { 12, T_1361 }, { 13, T_SRGB }, { 14, T_709 }, { 15, T_709 },
	                         { 8, T_LINEAR }, { 9, T_LOG100 }, { 10, T_LOG316 }, { 16, T_2084 }, { 17, T_428 },
	                         { 18, T_B67 } },
	             "unrecognized transfer characteristics");
	s.p = lookup(primaries, { { 4, P_470M }, { 5, P_470BG }, { 1, P_709 }, { 2, P_UNSPEC }, { 6, P_SMPTE_C },
	                          { 7, P_SMPTE_C }, { 8, P_FILM }, { 9, P_2020 }, { 10, P_XYZ }, { 11, P_DCI_P3 },
	                          { 12, P_DCI_P3_D65 }, { 22, P_EBU_3213_E } },
	             "unrecognized color primaries");
	return s;
}

Plan make_plan(Space in, Space out, double peak, bool approx, bool scene, bool adapt)
{
	// SMPTE 240M transfer is read as BT.709 unless scene referred (colorspace.cpp:101-107)
	if (!scene) {
		if (in.t == T_240M)
			in.t = T_709;
		if (out.t == T_240M)
			out.t = T_709;
	}
	Plan plan;
	if (in == out)
		return plan;
	if (!valid(in) || !valid(out))
		throw Error(kErrNoColorspaceConversion, "invalid colorspace definition");
	// breadth-first search; the first path found is the one kept
	std::unordered_map<int, std::pair<Space, int>> parent;
	std::deque<Space> queue{ in };
	std::unordered_map<int, bool> seen{ { key_of(in), true } };
	bool found = false;
	while (!queue.empty()) {
		const Space v = queue.front();
		queue.pop_front();
		if (v == out) {
			found = true;
			break;
		}
		for (const Edge &e : neighbours(v)) {
			if (seen.count(key_of(e.to)))
				continue;
			seen[key_of(e.to)] = true;
			queue.push_back(e.to);
			parent[key_of(e.to)] = { v, e.step };
		}
	}
	if (!found)
		throw Error(kErrNoColorspaceConversion, "no path between colorspaces");
	std::vector<std::pair<Space, int>> rev;  // (from, step) back from out
	for (Space v = out; !(v == in);) {
		const auto &pr = parent.at(key_of(v));
		rev.push_back(pr);
		v = pr.first;
	}
	if (rev.size() > static_cast<size_t>(kMaxOps))
		throw Error(kErrLogic, "too many colorspace operations");
	for (size_t k = 0; k < rev.size(); ++k) {
		const auto &step = rev[rev.size() - 1 - k];
		const Space to = k + 1 < rev.size() ? rev[rev.size() - 2 - k].first : out;
		plan.ops[plan.num_ops++] = make_op(step.second, step.first, to, peak, approx, scene, adapt);
	}
	return plan;
}

} // namespace csp
} // namespace zg
