/*
 * zimg_gb300 — zimg's separable polyphase resize (ResizeImplH / ResizeImplV)
 * on one GB300 GPU, behind a plain C ABI.
 *
 * Every pointer passed to a *_process call is a DEVICE pointer on the GPU that
 * was current when the object was created; every size is in elements or bytes
 * as stated. Objects are immutable after creation, so several host threads may
 * share one object, each with its own stream (as zimg's graphs are shared,
 * graphapp.cpp:355-377). No call allocates device memory while processing; the
 * caller provides the scratch buffer whose size *_get_tmp_size reports, as
 * zimg_filter_graph_process does (zimg.h:494-507).
 *
 * Plane strides are in bytes and may be negative (bottom-up planes: line i at
 * data + i * stride, as zimg_image_buffer allows, zimg.h:387-433); their
 * magnitude must cover a line.
 *
 * Each declaration names the zimg interface it replaces (paths relative to the
 * zimg source tree).
 */
#ifndef ZIMG_GB300_H_
#define ZIMG_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define ZG_API __declspec(dllexport)
#else
#define ZG_API __attribute__((visibility("default")))
#endif

#define ZG_API_VERSION_MAJOR 1
#define ZG_API_VERSION_MINOR 0

/* Same layout as cudaStream_t; 0 is the legacy default stream. */
typedef struct CUstream_st *zg_stream;

/* Error codes: the values of zimg_error_code_e (zimg.h:79-121). */
typedef enum zg_error_code {
	ZG_ERROR_UNKNOWN = -1,
	ZG_ERROR_SUCCESS = 0,
	ZG_ERROR_OUT_OF_MEMORY = 1,
	ZG_ERROR_USER_CALLBACK_FAILED = 2,
	ZG_ERROR_LOGIC = (1 << 10),
	ZG_ERROR_GREYSCALE_SUBSAMPLING = ZG_ERROR_LOGIC + 1,
	ZG_ERROR_COLOR_FAMILY_MISMATCH = ZG_ERROR_LOGIC + 2,
	ZG_ERROR_IMAGE_NOT_DIVISIBLE = ZG_ERROR_LOGIC + 3,
	ZG_ERROR_BIT_DEPTH_OVERFLOW = ZG_ERROR_LOGIC + 4,
	ZG_ERROR_ILLEGAL_ARGUMENT = (2 << 10),
	ZG_ERROR_ENUM_OUT_OF_RANGE = ZG_ERROR_ILLEGAL_ARGUMENT + 1,
	ZG_ERROR_INVALID_IMAGE_SIZE = ZG_ERROR_ILLEGAL_ARGUMENT + 2,
	ZG_ERROR_UNSUPPORTED_OPERATION = (3 << 10),
	ZG_ERROR_UNSUPPORTED_SUBSAMPLING = ZG_ERROR_UNSUPPORTED_OPERATION + 1,
	ZG_ERROR_NO_COLORSPACE_CONVERSION = ZG_ERROR_UNSUPPORTED_OPERATION + 2,
	ZG_ERROR_NO_FIELD_PARITY_CONVERSION = ZG_ERROR_UNSUPPORTED_OPERATION + 3,
	ZG_ERROR_RESAMPLING_NOT_AVAILABLE = ZG_ERROR_UNSUPPORTED_OPERATION + 4
} zg_error_code;

/* Pixel types: the values of zimg_pixel_type_e (zimg.h:191-196). WORD and FLOAT resize. */
typedef enum zg_pixel_type {
	ZG_PIXEL_BYTE = 0,
	ZG_PIXEL_WORD = 1,
	ZG_PIXEL_HALF = 2,
	ZG_PIXEL_FLOAT = 3
} zg_pixel_type;

/* Resampling filters: the values of zimg_resample_filter_e (zimg.h:374-382). */
typedef enum zg_resample_filter {
	ZG_RESIZE_POINT = 0,
	ZG_RESIZE_BILINEAR = 1,
	ZG_RESIZE_BICUBIC = 2,
	ZG_RESIZE_SPLINE16 = 3,
	ZG_RESIZE_SPLINE36 = 4,
	ZG_RESIZE_SPLINE64 = 6,
	ZG_RESIZE_LANCZOS = 5,
	/* zimg's internal value (zimg.cpp:21): the graph unresizes instead
	 * (graphbuilder.cpp:753-800); only zg_graph_build accepts it */
	ZG_RESIZE_UNRESIZE = -1
} zg_resample_filter;

/* Arithmetic the planner may pick for a pass (see zg_resize_params.engine). */
typedef enum zg_engine {
	ZG_ENGINE_AUTO = 0,    /* autotuner's choice */
	ZG_ENGINE_CUDA = 1,    /* CUDA-core kernels only */
	ZG_ENGINE_TENSOR = 2   /* banded matrix products on the tensor cores where the conversion allows it */
} zg_engine;

/* ------------------------------------------------------------------ errors --
 * Replaces zimg_get_last_error / zimg_clear_last_error (zimg.h:120-151,
 * zimg.cpp:531-538): the code and message of the last failure on this thread.
 */
ZG_API zg_error_code zg_get_last_error(char *err_msg, size_t n);
ZG_API void zg_clear_last_error(void);

/* ------------------------------------------------------- depth conversion --
 * Replaces zimg's DepthConversion (src/zimg/depth/depth.h:29-53,
 * depth.cpp:43-66), the filter the graph inserts around resize when the
 * pixel type, depth or range changes (src/zimg/graph/graphbuilder.cpp:943-950).
 * One plane per object, device planes, whole planes per call, as the resize
 * objects. The conversion is zimg's choice for the two formats:
 *   mode 0: formats equal (zimg's PixelFormat ==, pixel.h:194-199): a copy;
 *   mode 1: integer to integer, both limited range, same luma/chroma, depth
 *           not reduced: left shift (depth_convert.cpp:14-21);
 *   mode 2: to FLOAT or HALF: x * scale + offset from integers, the value
 *           itself between HALF and FLOAT (depth_convert.cpp:23-57; HALF is
 *           IEEE binary16, rounded to nearest even);
 *   mode 3: otherwise, to an integer type: x * scale + offset plus the dither
 *           value, clamped, rounded to nearest even (dither.cpp:37-54).
 * scale and offset are zimg's (quantize.h:19-45). Results equal zimg's C path
 * (CPUClass::NONE) bit for bit. Dither NONE, ORDERED (zimg's 16x16 matrix,
 * variant chosen by `plane` mod 4, dither.cpp:137-210), RANDOM (zimg's 64x64
 * blue-noise matrix at the offsets chosen by `plane` mod 4,
 * dither.cpp:219-234) and ERROR_DIFFUSION (Floyd-Steinberg over the whole
 * plane, dither.cpp:59-85 and 291-345; one thread block per plane runs the
 * lines as a wavefront) are built. ERROR_DIFFUSION on a plane of more than
 * 32 x 32 lines whose width leaves no launch shape within a block's shared
 * memory (from about 18,000 to 32,000 columns, by height) returns
 * ZG_ERROR_UNSUPPORTED_OPERATION. A limited-range format below 8 bits returns
 * ZG_ERROR_BIT_DEPTH_OVERFLOW (depth.cpp:52-53), as does a depth beyond its
 * type. */
typedef enum zg_dither_type {
	ZG_DITHER_NONE = 0,
	ZG_DITHER_ORDERED = 1,
	ZG_DITHER_RANDOM = 2,
	ZG_DITHER_ERROR_DIFFUSION = 3
} zg_dither_type;

/* zimg's PixelFormat (src/zimg/common/pixel.h:135-181). depth 0 = the
 * type's full depth. */
typedef struct zg_pixel_format {
	zg_pixel_type type;
	unsigned depth;
	int fullrange;
	int chroma;
	int ycgco;
} zg_pixel_format;

typedef struct zg_depth_params {
	unsigned width, height;
	zg_pixel_format pixel_in, pixel_out;
	zg_dither_type dither_type;
	unsigned plane;  /* 0-3: the plane's index in its image (selects the dither table variant) */
} zg_depth_params;

typedef struct zg_depth zg_depth;

ZG_API zg_error_code zg_depth_create(const zg_depth_params *params, zg_depth **out);
ZG_API void zg_depth_free(zg_depth *d);
/* The conversion chosen (*mode as above). */
ZG_API zg_error_code zg_depth_get_info(const zg_depth *d, int *mode);
/* Convert one plane (device pointers; strides in bytes) on `stream`. Never
 * allocates and never synchronises. */
ZG_API zg_error_code zg_depth_process(const zg_depth *d, const void *src, ptrdiff_t src_stride, void *dst,
                                      ptrdiff_t dst_stride, zg_stream stream);

/* --------------------------------------------------------------- colorspace --
 * Replaces zimg's ColorspaceConversion (src/zimg/colorspace/colorspace.h:
 * 117-132, colorspace.cpp:94-121) and its filter's process: three FLOAT
 * planes (Y'CbCr with centred chroma, R'G'B', linear RGB, ICtCp, ... as the
 * colorspaces say) converted per pixel. Colorspaces are zimg's API codes
 * (zimg_matrix_coefficients_e, zimg_transfer_characteristics_e,
 * zimg_color_primaries_e, zimg.h:283-352), mapped as zimg.cpp:238-305 maps
 * them: a code outside 0..255 returns ZG_ERROR_ENUM_OUT_OF_RANGE, a code
 * zimg does not map, an invalid colorspace or a pair without a path
 * ZG_ERROR_NO_COLORSPACE_CONVERSION. The operations are zimg's (path search
 * colorspace_graph.cpp:197-245; matrices computed in double and rounded to
 * float; transfer functions gamma.cpp). Matrix steps round like zimg's C
 * path; transfer functions use CUDA's powf / logf / log10f / expf, whose
 * results may differ from the C library's by a few units in the last place,
 * so outputs agree with zimg's C path to within the error bound the tests
 * state, not bit for bit. */
typedef struct zg_colorspace_params {
	unsigned width, height;
	int matrix_in, transfer_in, primaries_in;
	int matrix_out, transfer_out, primaries_out;
	double peak_luminance;      /* cd/m^2 of SDR white for PQ / HLG; NaN: 100 */
	int approximate_gamma;      /* as zimg: display-referred HLG then uses the per-channel curve */
	int scene_referred;
	int chromatic_adaptation;   /* Bradford white-point adaptation between primaries */
} zg_colorspace_params;

typedef struct zg_colorspace zg_colorspace;

ZG_API zg_error_code zg_colorspace_create(const zg_colorspace_params *params, zg_colorspace **out);
ZG_API void zg_colorspace_free(zg_colorspace *c);
/* Number of per-pixel operations (0: the identity) and, when kinds is not
 * NULL, their kinds in order into kinds[6]: 0 3x3 matrix, 1 transfer
 * function, 2 HLG OOTF + OETF, 3 inverse HLG, 4 constant luminance to RGB,
 * 5 RGB to constant luminance. */
ZG_API zg_error_code zg_colorspace_get_info(const zg_colorspace *c, unsigned *num_ops, int *kinds);
/* Convert the three planes src[0..2] into dst[0..2] (device pointers, strides
 * in bytes; dst may equal src plane by plane). The identity copies when dst
 * differs from src. Never allocates and never synchronises. */
ZG_API zg_error_code zg_colorspace_process(const zg_colorspace *c, const void *const src[3],
                                           const ptrdiff_t src_stride[3], void *const dst[3],
                                           const ptrdiff_t dst_stride[3], zg_stream stream);

/* ----------------------------------------------------------------- unresize --
 * Replaces zimg's UnresizeConversion (src/zimg/unresize/unresize.h:96-114,
 * unresize.cpp:34-91): the least-squares inverse of a bilinear upsampling of
 * one FLOAT plane, up_width x up_height -> orig_width x orig_height (shifts
 * as zimg's). Results equal zimg's C path (CPUClass::NONE) bit for bit. An
 * axis with orig > up returns ZG_ERROR_RESAMPLING_NOT_AVAILABLE ("unresize can
 * not upscale", bilinear.cpp:109-110); an axis that keeps its size and has
 * no shift is skipped, as zimg does. */
typedef struct zg_unresize_params {
	unsigned up_width, up_height;
	unsigned orig_width, orig_height;
	double shift_w, shift_h;
} zg_unresize_params;

typedef struct zg_unresize zg_unresize;

ZG_API zg_error_code zg_unresize_create(const zg_unresize_params *params, zg_unresize **out);
ZG_API void zg_unresize_free(zg_unresize *u);
ZG_API zg_error_code zg_unresize_get_tmp_size(const zg_unresize *u, size_t *out);
/* Device planes of FLOAT samples; tmp as *_get_tmp_size asks (may be NULL
 * when it is 0). */
ZG_API zg_error_code zg_unresize_process(const zg_unresize *u, const void *src, ptrdiff_t src_stride, void *dst,
                                         ptrdiff_t dst_stride, void *tmp, zg_stream stream);

/* Health of the pipelined kernels on the current device: 0, or which
 * bounded wait ran out inside one. Bits 0-7: the chained u16 kernel's TMA
 * form (1: a group's copies never landed, 2: a buffer was never released,
 * 3: a ring too small for a group). Bits 8-15: the tcgen05 FP32 wide kernel,
 * 16 + cause (17: converter warps, tile or operand buffer; 18: producer,
 * stage never released; 19: MMA lane, operands, accumulator or completion;
 * 20: epilogue, accumulator never complete). -1 when the device words cannot
 * be read. Nonzero means a library fault, not a caller error; the outputs of
 * the launches involved are not valid. With reset != 0 the words are
 * cleared. No zimg counterpart (zimg has no asynchronous device work). */
ZG_API int zg_pipeline_status(int reset);

/* Test hook for the bounded waits of the chained u16 kernel's TMA form
 * (current device): from the next launch on, CTA 0's producer skips group
 * drop_group of its pipeline without arming that group's stage (-1: none),
 * and every wait of that kernel gives up after wait_ns nanoseconds (0: the
 * default 0.25 s). A consumer wait then runs out, the kernel returns and
 * zg_pipeline_status reports cause 1. Returns 0, or -1 when the device
 * words cannot be written. Not for production use; no zimg counterpart. */
ZG_API int zg_debug_pipeline_fault(int drop_group, unsigned long long wait_ns);

/* The forms that ran the FP32 wide-filter passes enqueued by this host
 * thread since the last reset: bit 0 the mma.sync form (3xTF32 fragments in
 * registers), bit 1 the tcgen05 form (TMEM accumulators; vertical passes
 * whose tiles fill the SMs). With reset != 0 the mask is cleared after it is
 * read. A diagnostic for tests and tuning; no zimg counterpart. */
ZG_API int zg_wide_forms_used(int reset);

/* Version of this library. Replaces zimg_get_version_info (zimg.h:54). */
ZG_API void zg_get_version_info(unsigned *major, unsigned *minor, unsigned *micro);

/* --------------------------------------------------------- filter context --
 * Replaces compute_filter (src/zimg/resize/filter.h:178, filter.cpp:249-306):
 * the FP64 filter matrix, quantised to float and to signed 1.14 int16 taps
 * with zimg's error diffusion and row-sum fix-up (filter.cpp:43-127). Host
 * only; no GPU is touched. Call with f32 == NULL to learn *filter_width and
 * *filter_rows; then pass f32[rows*width], i16[rows*width], left[rows] (rows
 * packed without zimg's stride padding). width <= 0 means "src_dim".
 */
ZG_API zg_error_code zg_compute_filter(zg_resample_filter filter, double param_a, double param_b,
                                unsigned src_dim, unsigned dst_dim, double shift, double width,
                                unsigned *filter_width, unsigned *filter_rows,
                                float *f32, int16_t *i16, unsigned *left);

/* -------------------------------------------------------------- one pass --
 * Replaces ResizeImplBuilder{src_w, src_h, type}.set_horizontal()
 * .set_dst_dim().set_depth().set_filter().set_shift().set_subwidth().create()
 * (src/zimg/resize/resize_impl.h:45-63, resize_impl.cpp:245-267) and the
 * resulting filter's process() over every line (resize_impl.cpp:130-160).
 */
typedef struct zg_resize_pass zg_resize_pass;

typedef struct zg_pass_params {
	unsigned src_width;
	unsigned src_height;
	zg_pixel_type pixel_type;   /* WORD or FLOAT */
	unsigned depth;             /* bits per sample for WORD (1..16); ignored for FLOAT */
	int horizontal;             /* non-zero: ResizeImplH, else ResizeImplV */
	unsigned dst_dim;           /* output width (H) or height (V) */
	zg_resample_filter filter;
	double filter_param_a;      /* NaN: library default (zimg.cpp:320-350) */
	double filter_param_b;
	double shift;               /* in source pixels */
	double subwidth;            /* active source extent; <= 0 or NaN means src dim */
	zg_engine engine;
} zg_pass_params;

ZG_API zg_error_code zg_resize_pass_create(const zg_pass_params *params, zg_resize_pass **out);
ZG_API void zg_resize_pass_free(zg_resize_pass *pass);
/* Output plane size of the pass. */
ZG_API zg_error_code zg_resize_pass_get_output(const zg_resize_pass *pass, unsigned *width, unsigned *height);
/* Whole-plane process. Strides in bytes; src and dst must not overlap. */
ZG_API zg_error_code zg_resize_pass_process(const zg_resize_pass *pass, const void *src, ptrdiff_t src_stride,
                                     void *dst, ptrdiff_t dst_stride, zg_stream stream);

/* ----------------------------------------------------------- conversion --
 * Replaces ResizeConversion{w, h, type}.set_depth/filter/dst_width/dst_height/
 * shift_w/shift_h/subwidth/subheight/cpu().create() (src/zimg/resize/resize.h:
 * 22-44, resize.cpp:38-104): zero, one or two passes in zimg's order. The
 * planner fuses both passes into one kernel when the tile fits on chip, so
 * the intermediate plane never reaches HBM; otherwise the intermediate lives
 * in the caller's tmp buffer.
 */
typedef struct zg_resize zg_resize;

typedef struct zg_resize_params {
	unsigned src_width;
	unsigned src_height;
	zg_pixel_type pixel_type;
	unsigned depth;
	unsigned dst_width;
	unsigned dst_height;
	zg_resample_filter filter;
	double filter_param_a;
	double filter_param_b;
	double shift_w;
	double shift_h;
	double subwidth;            /* <= 0 or NaN: src_width */
	double subheight;           /* <= 0 or NaN: src_height */
	zg_engine engine;
	int allow_fusion;           /* 0: always two passes through tmp (testing) */
} zg_resize_params;

ZG_API void zg_resize_params_default(zg_resize_params *p);
ZG_API zg_error_code zg_resize_create(const zg_resize_params *params, zg_resize **out);
ZG_API void zg_resize_free(zg_resize *r);
/* Device scratch bytes that zg_resize_process needs (0 when fused or single pass). */
ZG_API zg_error_code zg_resize_get_tmp_size(const zg_resize *r, size_t *out);
/* Number of passes (0 = plain copy, 1, 2), whether the first is horizontal, and
 * how the passes run: 0 separate CUDA-core kernels, 1 one fused CUDA-core
 * kernel, 2 one fused tensor-core kernel, 3 separate kernels of which at least
 * one runs on the tensor cores (FP32 wide filters). */
ZG_API zg_error_code zg_resize_get_info(const zg_resize *r, int *num_passes, int *first_horizontal, int *fused);
ZG_API zg_error_code zg_resize_process(const zg_resize *r, const void *src, ptrdiff_t src_stride,
                                void *dst, ptrdiff_t dst_stride, void *tmp, zg_stream stream);

/*
 * No counterpart in zimg: zg_resize_process without a tmp argument, for
 * callers that cannot allocate device memory when they process a frame (a
 * plugin host that only hands out frame buffers from its own pool, a
 * real-time loop that must avoid cudaMalloc/cudaFree and their implicit
 * device-wide synchronisation). It allocates nothing: two-pass conversions
 * keep their intermediate plane in a scratch array compiled into the library,
 * ZG_NO_ALLOC_TMP_BYTES (32 MiB) per GPU, held until the process exits from
 * the time the library's module is loaded on that device (its first kernel
 * launch or symbol lookup there under CUDA's default lazy loading; context
 * creation under CUDA_MODULE_LOADING=EAGER, whether or not this entry point
 * is ever called). A conversion whose zg_resize_get_tmp_size exceeds
 * that is rejected with ZG_ERROR_OUT_OF_MEMORY and nothing is launched.
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture. All calls on a device share the one array, so
 * calls that overlap on the GPU (other streams, other threads) race; order
 * them on one stream or use zg_resize_process with separate tmp buffers.
 */
#define ZG_NO_ALLOC_TMP_BYTES ((size_t)32 << 20)
ZG_API zg_error_code zg_resize_process_no_alloc(const zg_resize *r, const void *src, ptrdiff_t src_stride,
                                                void *dst, ptrdiff_t dst_stride, zg_stream stream);

/* ---------------------------------------------------------------- batch --
 * Many planes of uneven sizes (luma plus subsampled chroma, mixed
 * resolutions) in one persistent launch. Replaces running one zimg graph per
 * frame on a thread pool (graphapp.cpp:355-425). Each job is a conversion as
 * in zg_resize_params. The caller fills a table of per-job device pointers
 * (zg_batch_io) once; zg_batch_process launches over the whole table, and
 * zg_batch_process_graph replays the same launch from a CUDA graph that the
 * batch captures on its first call on that stream.
 */
typedef struct zg_batch zg_batch;

typedef struct zg_batch_io {
	const void *src;
	ptrdiff_t src_stride;  /* bytes */
	void *dst;
	ptrdiff_t dst_stride;  /* bytes */
} zg_batch_io;

ZG_API zg_error_code zg_batch_create(const zg_resize_params *jobs, unsigned num_jobs, zg_batch **out);
ZG_API void zg_batch_free(zg_batch *b);
ZG_API zg_error_code zg_batch_get_tmp_size(const zg_batch *b, size_t *out);
/* Copy a host table of num_jobs entries into the batch's device table (async on stream). */
ZG_API zg_error_code zg_batch_set_io(zg_batch *b, const zg_batch_io *io, zg_stream stream);
/* One batch runs on one stream at a time: its launches share the batch's
 * device tables and work counter, so two zg_batch_process calls on the same
 * batch must not overlap (order them on one stream, or use two batches). */
ZG_API zg_error_code zg_batch_process(const zg_batch *b, void *tmp, zg_stream stream);
ZG_API zg_error_code zg_batch_process_graph(zg_batch *b, void *tmp, zg_stream stream);
/*
 * No counterpart in zimg (its CPU dispatch is fixed per build, cpuinfo.h):
 * the autotuner. For every set of jobs with identical parameters and engine
 * ZG_ENGINE_AUTO, times each distinct way the planner can run them (fused
 * CUDA-core kernel, separate CUDA-core passes, tensor-core kernel or passes)
 * as a batch of up to 16 of their bound planes (zg_batch_set_io first; their
 * outputs are overwritten with valid results), switches to the fastest when it
 * beats the planner's own choice by at least 5 %, and rebuilds the launch
 * groups. Allocates scratch for the trials and synchronises the stream. The
 * batch's tmp size may change: query zg_batch_get_tmp_size again. *changed
 * (optional) receives the number of jobs whose plan changed.
 */
ZG_API zg_error_code zg_batch_autotune(zg_batch *b, zg_stream stream, unsigned *changed);
/* Number of kernel launches one zg_batch_process issues. Where every chained
 * u16 job's source plane admits a tensor map (16-byte aligned base and
 * stride, set by zg_batch_set_io), the chained jobs of all kernel variants and
 * the identity planes run as one persistent launch whose CTAs take chunks of
 * work units from a counter (large chunks first, by estimated cost, small
 * ones last). */
ZG_API zg_error_code zg_batch_get_launch_count(const zg_batch *b, unsigned *out);

/* ---------------------------------------------------------------- graph --
 * Resize-only subset of zimg_filter_graph_build / _get_tmp_size / _process
 * (zimg.h:507,550-552,679; zimg.cpp:662-690). The format structs have the same
 * layout and meaning as zimg_image_format and zimg_graph_builder_params
 * (zimg.h:558-647), so a zimg caller's structs can be passed through after a
 * pointer cast. Supported: GREY/YUV/RGB with or without alpha, every pixel
 * type, changes of size, subsampling, pixel type, depth and range (the depth
 * conversions with the graph's dither type, placed as zimg places them,
 * graphbuilder.cpp:720-751,864-953); chroma siting, field parity and active
 * regions as zimg's graph builder maps them (graphbuilder.cpp:65-188,331-366,
 * 753-824). Alpha planes are full range in the integer types; straight alpha
 * through an interpolating resize is premultiplied in FLOAT 4:4:4 and divided
 * out afterwards, as zimg does (graphbuilder.cpp:594-600,1019-1068). A change
 * of matrix, transfer or primaries runs zimg's colorspace chain
 * (graphbuilder.cpp:975-1014): the colour planes to FLOAT 4:4:4 at the
 * smaller of the two geometries, the colorspace conversion (see
 * zg_colorspace_*), then each output plane to its geometry and format; GREY
 * to YUV / RGB without a conversion fills / duplicates the chroma planes and
 * YUV to GREY drops them. Colorspace codes zimg does not map, and pairs
 * without a path, return ZG_ERROR_NO_COLORSPACE_CONVERSION. A change of
 * alpha type, a colorspace change of an image with straight alpha, and
 * unresize of an image with straight alpha or with a colorspace change
 * return ZG_ERROR_UNSUPPORTED_OPERATION.
 */
typedef struct zg_image_format {
	unsigned version;
	unsigned width;
	unsigned height;
	int pixel_type;               /* zg_pixel_type */
	unsigned subsample_w;
	unsigned subsample_h;
	int color_family;             /* 0 GREY, 1 RGB, 2 YUV */
	int matrix_coefficients;
	int transfer_characteristics;
	int color_primaries;
	unsigned depth;
	int pixel_range;
	int field_parity;             /* 0 progressive, 1 top, 2 bottom */
	int chroma_location;          /* zimg_chroma_location_e values */
	struct {
		double left;
		double top;
		double width;
		double height;
	} active_region;
	int alpha;                    /* 0 none, 1 straight, 2 premultiplied */
} zg_image_format;

typedef struct zg_graph_builder_params {
	unsigned version;
	int resample_filter;          /* luma / RGB / alpha planes */
	double filter_param_a;
	double filter_param_b;
	int resample_filter_uv;       /* chroma planes */
	double filter_param_a_uv;
	double filter_param_b_uv;
	int dither_type;
	int cpu_type;
	double nominal_peak_luminance;
	char allow_approximate_gamma;
	char scene_referred;
	char chromatic_adaptation;
} zg_graph_builder_params;

/* Buffer descriptors as zimg_image_buffer(_const) (zimg.h:387-433): line i
 * of plane p at plane[p].data + (i & plane[p].mask) * plane[p].stride, in
 * device memory; mask = ZG_BUFFER_MAX for a whole plane, else 2^n - 1 for a
 * ring of 2^n lines (see zg_graph_process_cb). */
#define ZG_BUFFER_MAX (~0U)
typedef struct zg_image_buffer_const {
	unsigned version;
	struct {
		const void *data;
		ptrdiff_t stride;
		unsigned mask;
	} plane[4];
} zg_image_buffer_const;

typedef struct zg_image_buffer {
	unsigned version;
	struct {
		void *data;
		ptrdiff_t stride;
		unsigned mask;
	} plane[4];
} zg_image_buffer;

typedef struct zg_graph zg_graph;

/* API version numbers as ZIMG_MAKE_API_VERSION (zimg.h:30-38). */
#define ZG_MAKE_API_VERSION(x, y) (((x) << 8) | (y))
#define ZG_ZIMG_API_VERSION ZG_MAKE_API_VERSION(2, 4)

ZG_API void zg_image_format_default(zg_image_format *ptr, unsigned version);
ZG_API void zg_graph_builder_params_default(zg_graph_builder_params *ptr, unsigned version);
ZG_API zg_graph *zg_graph_build(const zg_image_format *src_format, const zg_image_format *dst_format,
                         const zg_graph_builder_params *params);
ZG_API void zg_graph_free(zg_graph *g);
ZG_API zg_error_code zg_graph_get_tmp_size(const zg_graph *g, size_t *out);
ZG_API zg_error_code zg_graph_process(const zg_graph *g, const zg_image_buffer_const *src, const zg_image_buffer *dst,
                               void *tmp, zg_stream stream);

/* Replaces zimg_filter_graph_callback and zimg_filter_graph_process with its
 * callbacks (zimg.h:455-484,550-552), and zimg_filter_graph_get_input/
 * output_buffering (zimg.h:522,534). Ring-buffer planes (mask != ZG_BUFFER_MAX)
 * go through whole-plane staging copies in tmp (zg_graph_get_tmp_size covers
 * them): for each step of input lines (the vertical subsampling unit, e.g. 2
 * for 4:2:0; i counts luma lines) unpack_cb(unpack_user, i, 0, width) is
 * called on the calling thread before those lines are read from the input
 * rings, and pack_cb(pack_user, i, 0, width) after output lines i .. i + step
 * - 1 have been written to the output rings and the stream has reached them;
 * a ring line is not overwritten before the callback that consumes or refills
 * it has returned. The callbacks are called for whole planes too; either may
 * be NULL. A callback that returns non-zero aborts processing with
 * ZG_ERROR_USER_CALLBACK_FAILED. The buffering queries return the smallest
 * ring (in luma lines, a power of 2) the graph accepts: the subsampling step. */
typedef int (*zg_graph_callback)(void *user, unsigned i, unsigned left, unsigned right);
ZG_API zg_error_code zg_graph_process_cb(const zg_graph *g, const zg_image_buffer_const *src,
                                         const zg_image_buffer *dst, void *tmp, zg_graph_callback unpack_cb,
                                         void *unpack_user, zg_graph_callback pack_cb, void *pack_user,
                                         zg_stream stream);
ZG_API zg_error_code zg_graph_get_input_buffering(const zg_graph *g, unsigned *out);
ZG_API zg_error_code zg_graph_get_output_buffering(const zg_graph *g, unsigned *out);
/* Per-plane resize parameters the builder chose (as zimg's FilterObserver
 * reports them, graphbuilder.h:45-64); returns 0 passes for a plane copied
 * unchanged. plane in 0..3. */
ZG_API zg_error_code zg_graph_get_plane_params(const zg_graph *g, int plane, zg_resize_params *out, int *present);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* ZIMG_GB300_H_ */
