// Colorspace conversion plan (zimg's ColorspaceConversion,
// src/zimg/colorspace/colorspace.cpp:94-121): the operations between two
// colorspaces, found on the host, run per pixel by colorspace_kernel.cu.
#pragma once

#include <cuda_runtime.h>

namespace zg {
namespace csp {

// zimg's internal enum orders (colorspace.h:19-60); the path search visits
// neighbours in this order.
enum Matrix : int { M_UNSPEC, M_RGB, M_601, M_709, M_FCC, M_240M, M_YCGCO, M_2020_NCL, M_2020_CL, M_CHROM_NCL,
                    M_CHROM_CL, M_LMS, M_ICTCP, M_COUNT };
enum Transfer : int { T_UNSPEC, T_LINEAR, T_LOG100, T_LOG316, T_709, T_470M, T_470BG, T_240M, T_XVYCC, T_1361,
                      T_SRGB, T_2084, T_428, T_B67, T_COUNT };
enum Primaries : int { P_UNSPEC, P_470M, P_470BG, P_SMPTE_C, P_709, P_FILM, P_2020, P_XYZ, P_DCI_P3, P_DCI_P3_D65,
                       P_EBU_3213_E, P_COUNT };

struct Space {
	int m, t, p;
	bool operator==(const Space &o) const { return m == o.m && t == o.t && p == o.p; }
};

enum OpKind : int { OP_MATRIX, OP_GAMMA, OP_HLG, OP_HLG_INV, OP_CL_TO_RGB, OP_CL_TO_YUV };

// One per-pixel operation; the fields a kind does not use are zero.
struct Op {
	int kind;
	int f, g;            // transfer function ids: GAMMA f; CL_TO_RGB f to linear; CL_TO_YUV f to gamma
	float m[3][3];       // MATRIX
	float pre, post;     // GAMMA: post * f(x * pre)
	float kr, kg, kb;    // luma weights (HLG, CL)
	float scale;         // HLG, CL
	float nb, pb, nr, pr;  // CL chroma scales
};

constexpr int kMaxOps = 6;

struct Plan {
	int num_ops = 0;
	Op ops[kMaxOps];
};

// zimg API codes (zimg_matrix_coefficients_e, ..._transfer_..., ..._primaries_e)
// to the internal enums, as zimg.cpp:238-305 maps them: outside 0..255
// ZG_ERROR_ENUM_OUT_OF_RANGE, unmapped ZG_ERROR_NO_COLORSPACE_CONVERSION
// (both thrown as zg::Error).
Space from_api(int matrix, int transfer, int primaries);

// The operations from `in` to `out`; empty when the colorspaces are equal
// after zimg's reading of SMPTE 240M transfer as BT.709 when not scene
// referred. Throws ZG_ERROR_NO_COLORSPACE_CONVERSION without a path.
Plan make_plan(Space in, Space out, double peak_luminance, bool approximate_gamma, bool scene_referred,
               bool chromatic_adaptation);

struct Launch {
	const void *src[3];
	ptrdiff_t src_stride[3];
	void *dst[3];
	ptrdiff_t dst_stride[3];
	int width, height;
	int vec;  // every plane 16-byte aligned in base and stride
	Plan plan;
};

cudaError_t launch_colorspace(const Launch &L, cudaStream_t stream);

} // namespace csp
} // namespace zg
