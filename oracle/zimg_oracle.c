/*
 * ORACLE — test infrastructure only. Not part of the shipped library.
 *
 * A plain-C restatement of zimg's separable polyphase resize, used by the
 * tests (as the checker), by smoke() and by bench.py's CPU-baseline leg. The
 * product never links, imports or calls this file.
 *
 * What it restates (paths relative to the zimg source tree):
 *   - filter kernels                 src/zimg/resize/filter.cpp:132-246
 *   - round_halfup                   src/zimg/resize/filter.cpp:32-40
 *   - compute_filter                 src/zimg/resize/filter.cpp:249-306
 *   - RowMatrix write semantics      src/zimg/common/matrix.cpp:14-21,93-149
 *   - matrix_to_filter (f32 + i16)   src/zimg/resize/filter.cpp:43-127
 *   - C line kernels u16/f32 H/V     src/zimg/resize/resize_impl.cpp:31-114
 *   - pass order / skip rules        src/zimg/resize/resize.cpp:12-18,38-104
 * plus an FP64 reference (unquantised taps, FP64 accumulation, FP64
 * intermediate) that the reference does not expose.
 *
 * Build with -ffp-contract=off (oracle/Makefile) so that the taps do not depend
 * on multiply-add fusion.
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846

enum { K_POINT = 0, K_BILINEAR = 1, K_BICUBIC = 2, K_SPLINE16 = 3, K_SPLINE36 = 4, K_LANCZOS = 5, K_SPLINE64 = 6 };

typedef struct {
	int kind;
	unsigned support;
	unsigned taps;
	double p0, p2, p3, q0, q1, q2, q3;
} orc_filter;

/* filter.cpp:21-30 */
static double orc_sinc(double x)
{
	return x == 0.0 ? 1.0 : sin(x * ORC_PI) / (x * ORC_PI);
}

static double orc_poly3(double x, double c0, double c1, double c2, double c3)
{
	return c0 + x * (c1 + x * (c2 + x * c3));
}

/* filter.cpp:32-40 */
static double orc_round_halfup(double x)
{
	return x < 0 ? floor(x + 0.5) : floor(x + 0.49999999999999994);
}

/* Filter construction with the API's NaN defaults (zimg.cpp:320-350). Returns 0 or -1 (illegal). */
int orc_filter_init(orc_filter *f, int kind, double a, double b)
{
	memset(f, 0, sizeof(*f));
	f->kind = kind;
	switch (kind) {
	case K_POINT: f->support = 0; return 0;
	case K_BILINEAR: f->support = 1; return 0;
	case K_BICUBIC: {
		/* filter.cpp:147-155 */
		double bb = isnan(a) ? 0.0 : a;
		double cc = isnan(b) ? 0.5 : b;
		f->p0 = (6.0 - 2.0 * bb) / 6.0;
		f->p2 = (-18.0 + 12.0 * bb + 6.0 * cc) / 6.0;
		f->p3 = (12.0 - 9.0 * bb - 6.0 * cc) / 6.0;
		f->q0 = (8.0 * bb + 24.0 * cc) / 6.0;
		f->q1 = (-12.0 * bb - 48.0 * cc) / 6.0;
		f->q2 = (6.0 * bb + 30.0 * cc) / 6.0;
		f->q3 = (-bb - 6.0 * cc) / 6.0;
		f->support = 2;
		return 0;
	}
	case K_SPLINE16: f->support = 2; return 0;
	case K_SPLINE36: f->support = 3; return 0;
	case K_SPLINE64: f->support = 4; return 0;
	case K_LANCZOS: {
		/* zimg.cpp:343-345 and filter.cpp:232-238 */
		double t = isnan(a) ? 3.0 : (a < 1.0 ? 1.0 : (a > 4294967295.0 ? 4294967295.0 : a));
		unsigned taps = (unsigned)t;
		if (taps >= 16)
			return -1;
		f->taps = taps;
		f->support = taps;
		return 0;
	}
	default:
		return -2;
	}
}

double orc_filter_eval(const orc_filter *f, double x)
{
	switch (f->kind) {
	case K_POINT:
		return 1.0;
	case K_BILINEAR: {
		double v = 1.0 - fabs(x);
		return v > 0.0 ? v : 0.0;
	}
	case K_BICUBIC:
		x = fabs(x);
		if (x < 1.0)
			return orc_poly3(x, f->p0, 0.0, f->p2, f->p3);
		else if (x < 2.0)
			return orc_poly3(x, f->q0, f->q1, f->q2, f->q3);
		return 0.0;
	case K_SPLINE16:
		x = fabs(x);
		if (x < 1.0)
			return orc_poly3(x, 1.0, -1.0 / 5.0, -9.0 / 5.0, 1.0);
		if (x < 2.0) {
			x -= 1.0;
			return orc_poly3(x, 0.0, -7.0 / 15.0, 4.0 / 5.0, -1.0 / 3.0);
		}
		return 0.0;
	case K_SPLINE36:
		x = fabs(x);
		if (x < 1.0)
			return orc_poly3(x, 1.0, -3.0 / 209.0, -453.0 / 209.0, 13.0 / 11.0);
		if (x < 2.0) {
			x -= 1.0;
			return orc_poly3(x, 0.0, -156.0 / 209.0, 270.0 / 209.0, -6.0 / 11.0);
		}
		if (x < 3.0) {
			x -= 2.0;
			return orc_poly3(x, 0.0, 26.0 / 209.0, -45.0 / 209.0, 1.0 / 11.0);
		}
		return 0.0;
	case K_SPLINE64:
		x = fabs(x);
		if (x < 1.0)
			return orc_poly3(x, 1.0, -3.0 / 2911.0, -6387.0 / 2911.0, 49.0 / 41.0);
		if (x < 2.0) {
			x -= 1.0;
			return orc_poly3(x, 0.0, -2328.0 / 2911.0, 4032.0 / 2911.0, -24.0 / 41.0);
		}
		if (x < 3.0) {
			x -= 2.0;
			return orc_poly3(x, 0.0, 582.0 / 2911.0, -1008.0 / 2911.0, 6.0 / 41.0);
		}
		if (x < 4.0) {
			x -= 3.0;
			return orc_poly3(x, 0.0, -97.0 / 2911.0, 168.0 / 2911.0, -1.0 / 41.0);
		}
		return 0.0;
	case K_LANCZOS:
		x = fabs(x);
		return x < f->taps ? orc_sinc(x) * orc_sinc(x / f->taps) : 0.0;
	default:
		return 0.0;
	}
}

/*
 * One dense row of the sparse matrix with RowMatrix's storage rule: a write
 * that does not change the stored value does not grow the row
 * (matrix.cpp:14-21); growing fills with zeros (matrix.cpp:103-129).
 */
typedef struct {
	double *buf; /* dense, indexed by column; zero outside [lo, hi) */
	size_t lo, hi;
	int empty;
} orc_row;

static double row_val(const orc_row *r, size_t j)
{
	return (r->empty || j < r->lo || j >= r->hi) ? 0.0 : r->buf[j];
}

static void row_assign(orc_row *r, size_t j, double v)
{
	if (row_val(r, j) == v)
		return;
	if (r->empty) {
		r->lo = j;
		r->hi = j + 1;
		r->empty = 0;
	} else if (j < r->lo) {
		r->lo = j;
	} else if (j >= r->hi) {
		r->hi = j + 1;
	}
	r->buf[j] = v;
}

/*
 * compute_filter + matrix_to_filter. Outputs rows*width taps packed densely.
 * Call with out_f32 == NULL to learn the shape. f64 (optional) receives the
 * unquantised matrix entries under the same window. Returns 0, or
 *   -1 illegal filter, -2 filter too wide, -3 out of memory.
 */
int orc_compute_filter(int kind, double a, double b, unsigned src_dim, unsigned dst_dim, double shift, double width,
                       unsigned *out_width, unsigned *out_rows,
                       float *out_f32, int16_t *out_i16, unsigned *out_left, double *out_f64)
{
	orc_filter f;
	if (orc_filter_init(&f, kind, a, b))
		return -1;

	double scale = (double)dst_dim / width;
	double step = scale < 1.0 ? scale : 1.0;
	double support = (double)f.support / step;
	unsigned filter_size = (unsigned)ceil(support) * 2U;
	if (filter_size < 1U)
		filter_size = 1U;
	if (support > (double)(unsigned)(UINT_MAX / 2))
		return -2;

	size_t rows = dst_dim;
	double *dense = calloc(src_dim ? src_dim : 1, sizeof(double));
	double **rowdata = calloc(rows ? rows : 1, sizeof(double *));
	size_t *lo = calloc(rows ? rows : 1, sizeof(size_t));
	size_t *hi = calloc(rows ? rows : 1, sizeof(size_t));
	int rc = 0;
	if (!dense || !rowdata || !lo || !hi) {
		rc = -3;
		goto done;
	}

	double src_hi = nextafter((double)src_dim, -INFINITY);
	for (unsigned i = 0; i < dst_dim; ++i) {
		orc_row r = { dense, 0, 0, 1 };
		/* filter.cpp:262-300 */
		double pos = (i + 0.5) / scale + shift;
		double begin_pos = orc_round_halfup(pos - filter_size / 2.0) + 0.5;

		double total = 0.0;
		for (unsigned j = 0; j < filter_size; ++j) {
			double xpos = begin_pos + j;
			total += orc_filter_eval(&f, (xpos - pos) * step);
		}

		size_t left = SIZE_MAX;
		for (unsigned j = 0; j < filter_size; ++j) {
			double xpos = begin_pos + j;
			double real_pos;
			if (xpos < 0.0)
				real_pos = -xpos;
			else if (xpos >= src_dim)
				real_pos = 2.0 * src_dim - xpos;
			else
				real_pos = xpos;
			if (real_pos < 0.0)
				real_pos = 0.0;
			if (real_pos > src_hi)
				real_pos = src_hi;

			size_t idx = (size_t)floor(real_pos);
			row_assign(&r, idx, row_val(&r, idx) + orc_filter_eval(&f, (xpos - pos) * step) / total);
			if (idx < left)
				left = idx;
		}
		if (row_val(&r, left) == 0.0) {
			row_assign(&r, left, DBL_EPSILON);
			row_assign(&r, left, 0.0);
		}

		lo[i] = r.lo;
		hi[i] = r.hi;
		rowdata[i] = malloc((r.hi - r.lo) * sizeof(double));
		if (!rowdata[i]) {
			rc = -3;
			goto done;
		}
		memcpy(rowdata[i], dense + r.lo, (r.hi - r.lo) * sizeof(double));
		memset(dense + r.lo, 0, (r.hi - r.lo) * sizeof(double));
	}

	/* matrix_to_filter (filter.cpp:43-127) */
	size_t fw = 0;
	for (size_t i = 0; i < rows; ++i)
		if (hi[i] - lo[i] > fw)
			fw = hi[i] - lo[i];
	*out_width = (unsigned)fw;
	*out_rows = (unsigned)rows;
	if (!out_f32)
		goto done;

	for (size_t i = 0; i < rows; ++i) {
		size_t left = lo[i] < (size_t)src_dim - fw ? lo[i] : (size_t)src_dim - fw;
		double f32_err = 0.0;
		double i16_err = 0.0;
		int16_t i16_sum = 0;
		int16_t i16_greatest = 0;
		size_t i16_greatest_idx = 0;

		for (size_t j = 0; j < fw; ++j) {
			size_t col = left + j;
			double coeff = (col < lo[i] || col >= hi[i]) ? 0.0 : rowdata[i][col - lo[i]];
			double expected_f32 = coeff - f32_err;
			double expected_i16 = coeff * (1 << 14) - i16_err;
			float c32 = (float)expected_f32;
			int16_t c16 = (int16_t)lrint(expected_i16);
			f32_err = (double)c32 - expected_f32;
			i16_err = (double)c16 - expected_i16;
			if (abs(c16) > abs(i16_greatest)) {
				i16_greatest = c16;
				i16_greatest_idx = j;
			}
			i16_sum = (int16_t)(i16_sum + c16);
			out_f32[i * fw + j] = c32;
			out_i16[i * fw + j] = c16;
			if (out_f64)
				out_f64[i * fw + j] = coeff;
		}
		out_i16[i * fw + i16_greatest_idx] = (int16_t)(out_i16[i * fw + i16_greatest_idx] + ((1 << 14) - i16_sum));
		out_left[i] = (unsigned)left;
	}

done:
	if (rowdata)
		for (size_t i = 0; i < rows; ++i)
			free(rowdata[i]);
	free(rowdata);
	free(lo);
	free(hi);
	free(dense);
	return rc;
}

/* ------------------------------------------------------------------ passes -- */

typedef struct {
	unsigned width, rows;
	float *f32;
	int16_t *i16;
	double *f64;
	unsigned *left;
} orc_ctx;

static void ctx_free(orc_ctx *c)
{
	free(c->f32);
	free(c->i16);
	free(c->f64);
	free(c->left);
	memset(c, 0, sizeof(*c));
}

static int ctx_make(orc_ctx *c, int kind, double a, double b, unsigned src_dim, unsigned dst_dim, double shift, double width)
{
	memset(c, 0, sizeof(*c));
	int rc = orc_compute_filter(kind, a, b, src_dim, dst_dim, shift, width, &c->width, &c->rows, NULL, NULL, NULL, NULL);
	if (rc)
		return rc;
	size_t n = (size_t)c->width * c->rows;
	c->f32 = malloc(n * sizeof(float) + 1);
	c->i16 = malloc(n * sizeof(int16_t) + 1);
	c->f64 = malloc(n * sizeof(double) + 1);
	c->left = malloc(c->rows * sizeof(unsigned) + 1);
	if (!c->f32 || !c->i16 || !c->f64 || !c->left) {
		ctx_free(c);
		return -3;
	}
	return orc_compute_filter(kind, a, b, src_dim, dst_dim, shift, width, &c->width, &c->rows, c->f32, c->i16, c->left, c->f64);
}

/* resize_impl.cpp:31-42. Arithmetic in uint32 mirrors int32 wraparound. */
static uint16_t pack_u16(uint32_t acc, int32_t pixel_max)
{
	int32_t x = (int32_t)(acc + (1u << 13));
	x = (x >> 14) + 32768;
	if (x > pixel_max)
		x = pixel_max;
	if (x < 0)
		x = 0;
	return (uint16_t)x;
}

enum { T_U16 = 1, T_F32 = 3, T_F64 = 4 };

typedef struct {
	const orc_ctx *ctx;
	int horizontal;
	int type;      /* T_U16, T_F32, T_F64 (T_F64: double in/out, f64 taps) */
	int use_fma;   /* f32 only */
	int32_t pixel_max;
	const void *src;
	ptrdiff_t src_stride; /* elements */
	void *dst;
	ptrdiff_t dst_stride; /* elements */
	unsigned out_w, out_h;
	unsigned row_begin, row_end;
} orc_job;

/* resize_line_{h,v}_{u16,f32}_c (resize_impl.cpp:44-114), one output row. */
static void run_row(const orc_job *job, unsigned i)
{
	const orc_ctx *c = job->ctx;
	unsigned fw = c->width;
	if (job->horizontal) {
		for (unsigned j = 0; j < job->out_w; ++j) {
			unsigned l = c->left[j];
			if (job->type == T_U16) {
				const uint16_t *s = (const uint16_t *)job->src + (ptrdiff_t)i * job->src_stride;
				uint32_t acc = 0;
				for (unsigned k = 0; k < fw; ++k)
					acc += (uint32_t)((int32_t)c->i16[(size_t)j * fw + k] * ((int32_t)s[l + k] - 32768));
				((uint16_t *)job->dst)[(ptrdiff_t)i * job->dst_stride + j] = pack_u16(acc, job->pixel_max);
			} else if (job->type == T_F32) {
				const float *s = (const float *)job->src + (ptrdiff_t)i * job->src_stride;
				float acc = 0;
				for (unsigned k = 0; k < fw; ++k)
					acc = job->use_fma ? fmaf(c->f32[(size_t)j * fw + k], s[l + k], acc) : acc + c->f32[(size_t)j * fw + k] * s[l + k];
				((float *)job->dst)[(ptrdiff_t)i * job->dst_stride + j] = acc;
			} else {
				const double *s = (const double *)job->src + (ptrdiff_t)i * job->src_stride;
				double acc = 0;
				for (unsigned k = 0; k < fw; ++k)
					acc += c->f64[(size_t)j * fw + k] * s[l + k];
				((double *)job->dst)[(ptrdiff_t)i * job->dst_stride + j] = acc;
			}
		}
	} else {
		unsigned top = c->left[i];
		if (job->type == T_U16) {
			const int16_t *co = c->i16 + (size_t)i * fw;
			for (unsigned j = 0; j < job->out_w; ++j) {
				uint32_t acc = 0;
				for (unsigned k = 0; k < fw; ++k) {
					const uint16_t *s = (const uint16_t *)job->src + (ptrdiff_t)(top + k) * job->src_stride;
					acc += (uint32_t)((int32_t)co[k] * ((int32_t)s[j] - 32768));
				}
				((uint16_t *)job->dst)[(ptrdiff_t)i * job->dst_stride + j] = pack_u16(acc, job->pixel_max);
			}
		} else if (job->type == T_F32) {
			const float *co = c->f32 + (size_t)i * fw;
			for (unsigned j = 0; j < job->out_w; ++j) {
				float acc = 0;
				for (unsigned k = 0; k < fw; ++k) {
					const float *s = (const float *)job->src + (ptrdiff_t)(top + k) * job->src_stride;
					acc = job->use_fma ? fmaf(co[k], s[j], acc) : acc + co[k] * s[j];
				}
				((float *)job->dst)[(ptrdiff_t)i * job->dst_stride + j] = acc;
			}
		} else {
			const double *co = c->f64 + (size_t)i * fw;
			for (unsigned j = 0; j < job->out_w; ++j) {
				double acc = 0;
				for (unsigned k = 0; k < fw; ++k) {
					const double *s = (const double *)job->src + (ptrdiff_t)(top + k) * job->src_stride;
					acc += co[k] * s[j];
				}
				((double *)job->dst)[(ptrdiff_t)i * job->dst_stride + j] = acc;
			}
		}
	}
}

static void *run_rows(void *arg)
{
	const orc_job *job = arg;
	for (unsigned i = job->row_begin; i < job->row_end; ++i)
		run_row(job, i);
	return NULL;
}

static int run_pass(const orc_job *proto, int nthreads)
{
	if (nthreads < 1)
		nthreads = 1;
	if (nthreads > 256)
		nthreads = 256;
	if ((unsigned)nthreads > proto->out_h)
		nthreads = proto->out_h ? (int)proto->out_h : 1;
	orc_job jobs[256];
	pthread_t th[256];
	int joined[256] = { 0 };
	unsigned per = (proto->out_h + nthreads - 1) / nthreads;
	for (int t = 0; t < nthreads; ++t) {
		jobs[t] = *proto;
		jobs[t].row_begin = t * per < proto->out_h ? t * per : proto->out_h;
		jobs[t].row_end = (t + 1) * per < proto->out_h ? (t + 1) * per : proto->out_h;
		if (t == 0)
			continue;
		if (pthread_create(&th[t], NULL, run_rows, &jobs[t]) == 0)
			joined[t] = 1;
		else
			run_rows(&jobs[t]);
	}
	run_rows(&jobs[0]);
	for (int t = 1; t < nthreads; ++t)
		if (joined[t])
			pthread_join(th[t], NULL);
	return 0;
}

/* resize.cpp:12-18 */
int orc_resize_h_first(double xscale, double yscale)
{
	double h_first_cost = (xscale > 1.0 ? xscale : 1.0) * 2.0 + xscale * (yscale > 1.0 ? yscale : 1.0);
	double v_first_cost = (yscale > 1.0 ? yscale : 1.0) + yscale * (xscale > 1.0 ? xscale : 1.0) * 2.0;
	return h_first_cost < v_first_cost;
}

/*
 * Pass list of ResizeConversion::create (resize.cpp:38-104):
 * returns the number of passes (0, 1, 2) and writes 1 for horizontal, 0 for
 * vertical into order[0..n).
 */
int orc_plan_order(unsigned src_w, unsigned src_h, unsigned dst_w, unsigned dst_h,
                   double shift_w, double shift_h, double subwidth, double subheight, int *order)
{
	int skip_h = (src_w == dst_w && shift_w == 0 && subwidth == src_w);
	int skip_v = (src_h == dst_h && shift_h == 0 && subheight == src_h);
	if (skip_h && skip_v)
		return 0;
	if (skip_h) {
		order[0] = 0;
		return 1;
	}
	if (skip_v) {
		order[0] = 1;
		return 1;
	}
	int h_first = orc_resize_h_first((double)dst_w / subwidth, (double)dst_h / subheight);
	order[0] = h_first ? 1 : 0;
	order[1] = h_first ? 0 : 1;
	return 2;
}

static size_t type_size(int type)
{
	return type == T_U16 ? 2 : (type == T_F32 ? 4 : 8);
}

/*
 * Whole-plane resize. type: 1 = u16 (C path, exact), 3 = f32 (sequential,
 * optionally fused multiply-add), 4 = FP64 oracle (double in/out).
 * Strides are in elements. Returns 0 or a negative error.
 */
int orc_resize_plane(int type, unsigned depth, int kind, double a, double b,
                     unsigned src_w, unsigned src_h, unsigned dst_w, unsigned dst_h,
                     double shift_w, double shift_h, double subwidth, double subheight,
                     int use_fma, int nthreads,
                     const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride)
{
	int order[2];
	int n = orc_plan_order(src_w, src_h, dst_w, dst_h, shift_w, shift_h, subwidth, subheight, order);
	size_t ts = type_size(type);
	if (n == 0) {
		for (unsigned i = 0; i < dst_h; ++i)
			memcpy((char *)dst + (size_t)i * dst_stride * ts, (const char *)src + (size_t)i * src_stride * ts, (size_t)dst_w * ts);
		return 0;
	}

	unsigned cur_w = src_w, cur_h = src_h;
	const void *cur = src;
	ptrdiff_t cur_stride = src_stride;
	void *tmp = NULL;
	int rc = 0;
	for (int p = 0; p < n; ++p) {
		int h = order[p];
		orc_ctx ctx;
		rc = h ? ctx_make(&ctx, kind, a, b, cur_w, dst_w, shift_w, subwidth)
		       : ctx_make(&ctx, kind, a, b, cur_h, dst_h, shift_h, subheight);
		if (rc)
			break;
		unsigned out_w = h ? dst_w : cur_w;
		unsigned out_h = h ? cur_h : dst_h;
		void *out;
		ptrdiff_t out_stride;
		if (p == n - 1) {
			out = dst;
			out_stride = dst_stride;
		} else {
			tmp = malloc((size_t)out_w * out_h * ts + 64);
			if (!tmp) {
				ctx_free(&ctx);
				rc = -3;
				break;
			}
			out = tmp;
			out_stride = out_w;
		}
		orc_job job;
		memset(&job, 0, sizeof(job));
		job.ctx = &ctx;
		job.horizontal = h;
		job.type = type;
		job.use_fma = use_fma;
		job.pixel_max = (int32_t)((1UL << depth) - 1);
		job.src = cur;
		job.src_stride = cur_stride;
		job.dst = out;
		job.dst_stride = out_stride;
		job.out_w = out_w;
		job.out_h = out_h;
		run_pass(&job, nthreads);
		ctx_free(&ctx);
		cur = out;
		cur_stride = out_stride;
		cur_w = out_w;
		cur_h = out_h;
	}
	free(tmp);
	return rc;
}

/*
 * A conversion planned once and run on many planes, as zimg's graph is built
 * once and then processes frames (graphapp.cpp:355-425): the filter contexts
 * of ResizeConversion's passes (resize.cpp:38-104) are computed at creation,
 * and each run resizes one plane on the calling thread, with the
 * intermediate plane in caller-provided scratch. This serves the CPU
 * baseline, which runs frames in parallel on every host thread.
 */
typedef struct orc_plan {
	int type, n, order[2], use_fma;
	unsigned depth, src_w, src_h, dst_w, dst_h, mid_w, mid_h;
	orc_ctx ctx[2];
} orc_plan;

void orc_plan_free(orc_plan *p)
{
	if (!p)
		return;
	for (int i = 0; i < p->n; ++i)
		ctx_free(&p->ctx[i]);
	free(p);
}

orc_plan *orc_plan_create(int type, unsigned depth, int kind, double a, double b,
                          unsigned src_w, unsigned src_h, unsigned dst_w, unsigned dst_h,
                          double shift_w, double shift_h, double subwidth, double subheight, int use_fma)
{
	orc_plan *p = calloc(1, sizeof(orc_plan));
	if (!p)
		return NULL;
	p->type = type;
	p->depth = depth;
	p->use_fma = use_fma;
	p->src_w = src_w;
	p->src_h = src_h;
	p->dst_w = dst_w;
	p->dst_h = dst_h;
	int n = orc_plan_order(src_w, src_h, dst_w, dst_h, shift_w, shift_h, subwidth, subheight, p->order);
	unsigned cur_w = src_w, cur_h = src_h;
	for (int i = 0; i < n; ++i) {
		int h = p->order[i];
		int rc = h ? ctx_make(&p->ctx[i], kind, a, b, cur_w, dst_w, shift_w, subwidth)
		           : ctx_make(&p->ctx[i], kind, a, b, cur_h, dst_h, shift_h, subheight);
		if (rc) {
			orc_plan_free(p);
			return NULL;
		}
		p->n = i + 1;
		if (h)
			cur_w = dst_w;
		else
			cur_h = dst_h;
		if (i == 0) {
			p->mid_w = cur_w;
			p->mid_h = cur_h;
		}
	}
	p->n = n;
	return p;
}

size_t orc_plan_tmp_size(const orc_plan *p)
{
	return p->n == 2 ? (size_t)p->mid_w * p->mid_h * type_size(p->type) : 0;
}

int orc_plan_run(const orc_plan *p, const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride, void *tmp)
{
	size_t ts = type_size(p->type);
	if (p->n == 0) {
		for (unsigned i = 0; i < p->dst_h; ++i)
			memcpy((char *)dst + (size_t)i * dst_stride * ts, (const char *)src + (size_t)i * src_stride * ts,
			       (size_t)p->dst_w * ts);
		return 0;
	}
	if (p->n == 2 && !tmp)
		return -1;
	unsigned cur_w = p->src_w, cur_h = p->src_h;
	const void *cur = src;
	ptrdiff_t cur_stride = src_stride;
	for (int i = 0; i < p->n; ++i) {
		int h = p->order[i];
		orc_job job;
		memset(&job, 0, sizeof(job));
		job.ctx = &p->ctx[i];
		job.horizontal = h;
		job.type = p->type;
		job.use_fma = p->use_fma;
		job.pixel_max = (int32_t)((1UL << p->depth) - 1);
		job.src = cur;
		job.src_stride = cur_stride;
		job.out_w = h ? p->dst_w : cur_w;
		job.out_h = h ? cur_h : p->dst_h;
		job.dst = i == p->n - 1 ? dst : tmp;
		job.dst_stride = i == p->n - 1 ? dst_stride : (ptrdiff_t)job.out_w;
		job.row_begin = 0;
		job.row_end = job.out_h;
		run_rows(&job);
		cur = job.dst;
		cur_stride = job.dst_stride;
		cur_w = job.out_w;
		cur_h = job.out_h;
	}
	return 0;
}

/* One pass (ResizeImplBuilder, resize_impl.cpp:245-267) on a whole plane. */
int orc_resize_pass(int type, unsigned depth, int horizontal, int kind, double a, double b,
                    unsigned src_w, unsigned src_h, unsigned dst_dim, double shift, double subwidth,
                    int use_fma, int nthreads,
                    const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride)
{
	orc_ctx ctx;
	int rc = ctx_make(&ctx, kind, a, b, horizontal ? src_w : src_h, dst_dim, shift, subwidth);
	if (rc)
		return rc;
	orc_job job;
	memset(&job, 0, sizeof(job));
	job.ctx = &ctx;
	job.horizontal = horizontal;
	job.type = type;
	job.use_fma = use_fma;
	job.pixel_max = (int32_t)((1UL << depth) - 1);
	job.src = src;
	job.src_stride = src_stride;
	job.dst = dst;
	job.dst_stride = dst_stride;
	job.out_w = horizontal ? dst_dim : src_w;
	job.out_h = horizontal ? src_h : dst_dim;
	run_pass(&job, nthreads);
	ctx_free(&ctx);
	return 0;
}

/* ------------------------------------------------------------------ depth --
 * zimg's depth conversion around resize (src/zimg/depth/), its C path
 * (CPUClass::NONE): DepthConversion::create (depth.cpp:52-66) picks a plain
 * copy, a lossless left shift (depth_convert.cpp:14-21), a conversion to float
 * (depth_convert.cpp:32-39) or a dither to integer (dither.cpp:37-54, types
 * NONE and ORDERED; RANDOM and ERROR_DIFFUSION are not restated). Pixel types
 * follow zimg.h (0 BYTE, 1 WORD, 2 HALF, 3 FLOAT).
 */
typedef struct orc_pixfmt {
	int type;
	unsigned depth;
	int fullrange, chroma, ycgco;
} orc_pixfmt;

static int pix_is_float(int t)
{
	return t == 2 || t == 3;
}

static size_t pix_size(int t)
{
	return t == 0 ? 1 : (t == 3 ? 4 : 2);
}

/* integer_offset / integer_range, quantize.h:19-32 */
static double pix_offset(const orc_pixfmt *f)
{
	if (pix_is_float(f->type))
		return 0.0;
	if (f->chroma)
		return (double)(1L << (f->depth - 1));
	if (!f->fullrange)
		return (double)(16L << (f->depth - 8));
	return 0.0;
}

static double pix_range(const orc_pixfmt *f)
{
	if (pix_is_float(f->type))
		return 1.0;
	if (f->fullrange)
		return (double)((1L << f->depth) - 1);
	if (f->chroma && !f->ycgco)
		return (double)(224L << (f->depth - 8));
	return (double)(219L << (f->depth - 8));
}

/* get_scale_offset, quantize.h:34-45: FP64, then rounded to float */
void orc_depth_scale_offset(const orc_pixfmt *in, const orc_pixfmt *out, float *scale, float *offset)
{
	double ri = pix_range(in), oi = pix_offset(in), ro = pix_range(out), oo = pix_offset(out);
	*scale = (float)(ro / ri);
	*offset = (float)(-oi * ro / ri + oo);
}

/* PixelFormat equality, common/pixel.h:194-199 */
static int pix_equal(const orc_pixfmt *a, const orc_pixfmt *b)
{
	if (pix_is_float(a->type))
		return a->type == b->type && a->chroma == b->chroma;
	return a->type == b->type && a->depth == b->depth && a->fullrange == b->fullrange && a->chroma == b->chroma;
}

/* The ordered-dither matrix of dither.cpp:137-155: a 16x16 Bayer matrix,
 * written here from its recursive definition rather than as a table: digit k
 * (k = 0 the least significant bit of the row i and the column j) contributes
 * B[bit_k(i)][bit_k(j)] * 4^(3-k), with B = {{0, 3}, {2, 1}}. */
unsigned orc_bayer16(unsigned i, unsigned j)
{
	static const unsigned B[2][2] = { { 0, 3 }, { 2, 1 } };
	unsigned v = 0;
	for (unsigned k = 0; k < 4; ++k)
		v += B[(i >> k) & 1][(j >> k) & 1] << (2 * (3 - k));
	return v;
}

/* zimg's 64 x 64 blue-noise matrix (blue.h:10-13): data without a generating
 * rule, read out of zimg's own build into the library's include file, which
 * packs four row-major entries per little-endian word. */
static const uint32_t orc_blue_noise_words[1024] = {
#include "../zimg_gb300/csrc/blue_noise_table.inc"
};

unsigned orc_blue_noise(unsigned i, unsigned j)
{
	const unsigned k = (i & 63) * 64 + (j & 63);
	return (orc_blue_noise_words[k >> 2] >> (8 * (k & 3))) & 0xFF;
}

/* Dither offset of row i, column j for plane `seq` (dither.cpp:157-234).
 * ORDERED (1): (m + 1) / 257 - 1/2 in float, from the Bayer matrix as is
 * (seq 0), mirrored left-right (1), top-bottom (2) or transposed (3).
 * RANDOM (2): the same mapping of the blue-noise entry at row (i + voff) mod
 * 64, column (j + hoff) mod 64, (hoff, voff) = (0, 0), (32, 12), (16, 55),
 * (48, 26) for seq mod 4 (dither.cpp:226-233). NONE (0): zero. */
float orc_dither_value(int dither, unsigned seq, unsigned i, unsigned j)
{
	if (dither == 0)
		return 0.0f;
	if (dither == 2) {
		static const unsigned hoff[4] = { 0, 32, 16, 48 }, voff[4] = { 0, 12, 55, 26 };
		const unsigned m = orc_blue_noise(i + voff[seq % 4], j + hoff[seq % 4]);
		return (float)(m + 1) / 257.0f - 0.5f;
	}
	i &= 15;
	j &= 15;
	unsigned m;
	switch (seq % 4) {
	case 0: m = orc_bayer16(i, j); break;
	case 1: m = orc_bayer16(i, 15 - j); break;
	case 2: m = orc_bayer16(15 - i, j); break;
	default: m = orc_bayer16(j, i); break;
	}
	return (float)(m + 1) / 257.0f - 0.5f;
}

/* IEEE binary16 <-> binary32 (quantize.cpp:24-146 follows the same
 * definitions): half to float is exact; float to half rounds to nearest
 * even, overflows to infinity, and keeps NaNs quiet with the payload's top
 * bits. Written here from the IEEE formats. */
float orc_half_to_float(uint16_t h)
{
	const uint32_t sign = (uint32_t)(h >> 15) << 31;
	const uint32_t e = (h >> 10) & 0x1F, m = h & 0x3FF;
	uint32_t bits;
	if (e == 0x1F) {
		bits = sign | 0x7F800000u | (m ? ((m << 13) | 0x00400000u) : 0);
	} else if (e == 0) {
		if (m == 0) {
			bits = sign;
		} else {
			/* subnormal: normalise the significand */
			int k = 0;
			uint32_t mm = m;
			while (!(mm & 0x400)) {
				mm <<= 1;
				++k;
			}
			bits = sign | ((uint32_t)(127 - 15 - k + 1) << 23) | ((mm & 0x3FF) << 13);
		}
	} else {
		bits = sign | ((e + 127 - 15) << 23) | (m << 13);
	}
	float f;
	memcpy(&f, &bits, 4);
	return f;
}

uint16_t orc_float_to_half(float f)
{
	uint32_t x;
	memcpy(&x, &f, 4);
	const uint32_t sign = (x >> 31) << 15;
	const uint32_t e = (x >> 23) & 0xFF, m = x & 0x7FFFFF;
	if (e == 0xFF)
		return (uint16_t)(sign | 0x7C00u | (m ? ((m >> 13) | 0x200u) : 0));
	/* the significand with its leading bit, and how far it must move right
	 * for a half's 10 stored bits (more for results below the normal range) */
	uint32_t sig = m, shift = 13, he;
	if (e <= 112) {
		shift = 13 + 112 - e + 1;
		if (shift > 31)
			shift = 31;
		sig = m | 0x800000u;
		he = 0;
	} else {
		he = e - 112;
	}
	/* round to nearest, ties to even */
	const uint32_t rem = sig & ((1u << shift) - 1), halfway = 1u << (shift - 1);
	uint32_t q = sig >> shift;
	if (rem > halfway || (rem == halfway && (q & 1)))
		++q;
	if (q > 0x3FF) {
		q &= 0x3FF;
		++he;
	}
	if (he >= 0x1F)
		return (uint16_t)(sign | 0x7C00u);
	return (uint16_t)(sign | (he << 10) | q);
}

static float load_sample(int type, const void *row, unsigned j)
{
	if (type == 0)
		return (float)((const uint8_t *)row)[j];
	if (type == 1)
		return (float)((const uint16_t *)row)[j];
	if (type == 2)
		return orc_half_to_float(((const uint16_t *)row)[j]);
	return ((const float *)row)[j];
}

/* Mode of a conversion (depth.cpp:52-66): 0 copy, 1 left shift, 2 to float
 * or half, 3 dither; negative: zimg's error (-1 bit depth below 8 in limited
 * range, -2 not restated here: RANDOM / ERROR_DIFFUSION dither). */
int orc_depth_mode(const orc_pixfmt *in, const orc_pixfmt *out, int dither)
{
	if ((!in->fullrange && in->depth < 8) || (!out->fullrange && out->depth < 8))
		return -1;
	if (pix_equal(in, out))
		return 0;
	if (!pix_is_float(in->type) && !pix_is_float(out->type) && !in->fullrange && !out->fullrange &&
	    in->chroma == out->chroma && out->depth >= in->depth)
		return 1;
	if (pix_is_float(out->type))
		return (pix_is_float(in->type) && in->type == out->type) ? 0 : 2;
	return (dither >= 0 && dither <= 3) ? 3 : -2;
}

/* Floyd-Steinberg error diffusion over a whole plane, zimg's C path
 * (dither.cpp:59-85 per row, rows in order with two error rows that swap,
 * dither.cpp:328-343). The error rows are padded by one zero on each side and
 * start at zero. Each sample: x = sample * scale + offset (two roundings),
 * then the error 0 + left * 7/16 + top-right * 3/16 + top * 5/16 +
 * top-left * 1/16 summed in that order, x + error, clamped to [0, 2^depth -
 * 1] (a NaN stays NaN), rounded to nearest even (a NaN gives 0), and the
 * sample's error x - q. */
static int orc_error_diffusion(const orc_pixfmt *in, const orc_pixfmt *out, float scale, float offset, unsigned w,
                               unsigned h, const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride)
{
	float *rows = calloc(2 * ((size_t)w + 2), sizeof(float));
	if (!rows)
		return -3;
	float *const err_a = rows, *const err_b = rows + w + 2;
	const float vmax = (float)((1UL << out->depth) - 1);
	for (unsigned i = 0; i < h; ++i) {
		const char *s = (const char *)src + (ptrdiff_t)i * src_stride;
		char *d = (char *)dst + (ptrdiff_t)i * dst_stride;
		const float *top = (i % 2) ? err_a : err_b;
		float *cur = (i % 2) ? err_b : err_a;
		for (unsigned j = 0; j < w; ++j) {
			const unsigned je = j + 1;
			const float p = load_sample(in->type, s, j) * scale;
			float x = p + offset;
			float err = 0.0f;
			err = err + cur[je - 1] * (7.0f / 16.0f);
			err = err + top[je + 1] * (3.0f / 16.0f);
			err = err + top[je + 0] * (5.0f / 16.0f);
			err = err + top[je - 1] * (1.0f / 16.0f);
			x = x + err;
			x = x < 0.0f ? 0.0f : (vmax < x ? vmax : x);
			const unsigned q = isnan(x) ? 0u : (unsigned)lrintf(x);
			if (out->type == 0)
				((uint8_t *)d)[j] = (uint8_t)q;
			else
				((uint16_t *)d)[j] = (uint16_t)q;
			cur[je] = x - (float)q;
		}
	}
	free(rows);
	return 0;
}

int orc_depth_convert(const orc_pixfmt *in, const orc_pixfmt *out, int dither, unsigned seq, unsigned w, unsigned h,
                      const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride)
{
	const int mode = orc_depth_mode(in, out, dither);
	if (mode < 0)
		return mode;
	float scale = 1.0f, offset = 0.0f;
	orc_depth_scale_offset(in, out, &scale, &offset);
	if (mode == 3 && dither == 3)
		return orc_error_diffusion(in, out, scale, offset, w, h, src, src_stride, dst, dst_stride);
	const unsigned shift = out->depth - in->depth;
	const float vmax = (float)((1UL << out->depth) - 1);
	for (unsigned i = 0; i < h; ++i) {
		const char *s = (const char *)src + (ptrdiff_t)i * src_stride;
		char *d = (char *)dst + (ptrdiff_t)i * dst_stride;
		for (unsigned j = 0; j < w; ++j) {
			if (mode == 0) {
				const size_t n = pix_size(out->type);
				memcpy(d + j * n, s + j * n, n);
			} else if (mode == 1) {
				/* integer_to_integer, depth_convert.cpp:14-21 */
				const unsigned x = in->type == 0 ? ((const uint8_t *)s)[j] : ((const uint16_t *)s)[j];
				if (out->type == 0)
					((uint8_t *)d)[j] = (uint8_t)(x << shift);
				else
					((uint16_t *)d)[j] = (uint16_t)(x << shift);
			} else if (mode == 2) {
				/* integer_to_float / integer_to_half (product, then sum), or
				 * half <-> float as is (depth_convert.cpp:23-57) */
				float v;
				if (pix_is_float(in->type)) {
					v = load_sample(in->type, s, j);
				} else {
					const float p = load_sample(in->type, s, j) * scale;
					v = p + offset;
				}
				if (out->type == 2)
					((uint16_t *)d)[j] = orc_float_to_half(v);
				else
					((float *)d)[j] = v;
			} else {
				/* dither_ordered, dither.cpp:37-54 */
				const float p = load_sample(in->type, s, j) * scale;
				float x = p + offset;
				x = x + orc_dither_value(dither, seq, i, j);
				x = x < 0.0f ? 0.0f : (vmax < x ? vmax : x);
				const long q = lrintf(x);
				if (out->type == 0)
					((uint8_t *)d)[j] = (uint8_t)q;
				else
					((uint16_t *)d)[j] = (uint16_t)q;
			}
		}
	}
	return 0;
}

/* ---------------------------------------------------------------- unresize --
 * zimg's unresize (src/zimg/unresize/): the least-squares inverse of a
 * bilinear upsampling, FP32 only, C path.
 *
 * Context (bilinear.cpp:60-170), all FP64: A (up x orig) holds the bilinear
 * weights of each upsampled sample, written with RowMatrix's rule (a write
 * that does not change the value does not grow the row); A' is its transpose
 * under the same rule, then trimmed of zeros at both ends (matrix.cpp:164-200);
 * of A'A (matrix.cpp:202-219: k ascending over A' row r's run, products then
 * sums) only the band r-1..r+1 is used, by a tridiagonal LU with DBL_EPSILON
 * guards (bilinear.cpp:20-57). The per-line data are A''s rows packed to a
 * common width (their run starts clamped so the run fits) and the LU terms
 * as float, 1/(l + eps) pre-inverted.
 */
typedef struct {
	unsigned up, orig;      /* input (upsampled) and output (original) dimensions */
	unsigned row_size;
	float *coef;            /* [orig][row_size] */
	unsigned *offset;       /* [orig] */
	float *lu_c, *lu_l, *lu_u;
} orc_unresize_ctx;

void orc_unresize_ctx_free(orc_unresize_ctx *c)
{
	free(c->coef);
	free(c->offset);
	free(c->lu_c);
	free(c->lu_l);
	free(c->lu_u);
	memset(c, 0, sizeof(*c));
}

/* A's row i: up to two (column, weight) entries (bilinear_weights,
 * bilinear.cpp:60-104, with shift already mapped to the input grid). */
static int bilinear_row(unsigned in, unsigned out, double shift, unsigned i, unsigned col[2], double w[2])
{
	const double leftmost = 0.5 + shift, rightmost = in - 0.5 + shift;
	double lf = floor(leftmost), rf = floor(rightmost);
	lf = lf < 0.0 ? 0.0 : (lf > in - 1.0 ? in - 1.0 : lf);
	rf = rf < 0.0 ? 0.0 : (rf > in - 1.0 ? in - 1.0 : rf);
	const double position = (i + 0.5) * in / out;
	int n = 0;
	if (position <= leftmost) {
		col[n] = (unsigned)lf;
		w[n++] = 1.0;
	} else if (position >= rightmost) {
		col[n] = (unsigned)rf;
		w[n++] = 1.0;
	} else {
		const unsigned left = (unsigned)floor(position - leftmost);
		const double distance = position - left - leftmost;
		/* a zero weight leaves the row as it is */
		if (1.0 - distance != 0.0) {
			col[n] = left;
			w[n++] = 1.0 - distance;
		}
		if (distance != 0.0) {
			col[n] = left + 1;
			w[n++] = distance;
		}
	}
	return n;
}

int orc_unresize_context(unsigned orig, unsigned up, double shift, orc_unresize_ctx *ctx)
{
	memset(ctx, 0, sizeof(*ctx));
	if (orig > up)
		return -2; /* "unresize can not upscale" */
	const unsigned N = orig, M = up;
	const double s = -shift * N / M; /* output shift mapped to the input grid */
	/* A as M rows of at most 2 entries */
	unsigned *acol = malloc(sizeof(unsigned) * 2 * M);
	double *aw = malloc(sizeof(double) * 2 * M);
	int *an = malloc(sizeof(int) * M);
	/* A' row r: run [lo, hi) over A's rows, lo the first row with a nonzero
	 * entry in column r, hi one past the last */
	size_t *lo = malloc(sizeof(size_t) * N), *hi = malloc(sizeof(size_t) * N);
	if (!acol || !aw || !an || !lo || !hi) {
		free(acol); free(aw); free(an); free(lo); free(hi);
		return -3;
	}
	for (unsigned r = 0; r < N; ++r) {
		lo[r] = 0;
		hi[r] = 0;
	}
	for (unsigned i = 0; i < M; ++i) {
		an[i] = bilinear_row(N, M, s, i, acol + 2 * i, aw + 2 * i);
		for (int e = 0; e < an[i]; ++e) {
			const unsigned r = acol[2 * i + e];
			if (hi[r] == 0) {
				lo[r] = i;
				hi[r] = i + 1;
			} else {
				hi[r] = i + 1;
			}
		}
	}
	/* A[i][c] */
#define A_AT(i, c) (an[i] > 0 && acol[2 * (i)] == (c) ? aw[2 * (i)] : (an[i] > 1 && acol[2 * (i) + 1] == (c) ? aw[2 * (i) + 1] : 0.0))
	/* band of A'A: P[r][c] = sum over k in A' row r's run of A'[r][k] * A[k][c] */
	double *pl = malloc(sizeof(double) * N), *pd = malloc(sizeof(double) * N), *pu = malloc(sizeof(double) * N);
	unsigned row_size = 0;
	for (unsigned r = 0; r < N; ++r) {
		double acc[3] = { 0.0, 0.0, 0.0 };
		for (int t = 0; t < 3; ++t) {
			const long c = (long)r - 1 + t;
			if (c < 0 || c >= (long)N)
				continue;
			double a = 0.0;
			for (size_t k = lo[r]; k < hi[r]; ++k) {
				const double p = A_AT(k, r) * A_AT(k, (unsigned)c);
				a = a + p;
			}
			acc[t] = a;
		}
		pl[r] = acc[0];
		pd[r] = acc[1];
		pu[r] = acc[2];
		if (hi[r] - lo[r] > row_size)
			row_size = (unsigned)(hi[r] - lo[r]);
	}
	/* tridiagonal LU (bilinear.cpp:20-57) */
	double *c = calloc(N, sizeof(double)), *l = calloc(N, sizeof(double)), *u = calloc(N, sizeof(double));
	const double eps = DBL_EPSILON;
	if (N == 1) {
		l[0] = pd[0];
	} else {
		c[0] = 0.0;
		l[0] = pd[0];
		u[0] = pu[0] / (pd[0] + eps);
		for (unsigned i = 1; i + 1 < N; ++i) {
			c[i] = pl[i];
			l[i] = pd[i] - c[i] * u[i - 1];
			u[i] = pu[i] / (l[i] + eps);
		}
		c[N - 1] = pl[N - 1];
		l[N - 1] = pd[N - 1] - c[N - 1] * u[N - 2];
		u[N - 1] = 0.0;
	}
	ctx->up = M;
	ctx->orig = N;
	ctx->row_size = row_size;
	ctx->coef = calloc((size_t)N * (row_size ? row_size : 1), sizeof(float));
	ctx->offset = calloc(N, sizeof(unsigned));
	ctx->lu_c = malloc(sizeof(float) * N);
	ctx->lu_l = malloc(sizeof(float) * N);
	ctx->lu_u = malloc(sizeof(float) * N);
	for (unsigned r = 0; r < N; ++r) {
		size_t left = lo[r] < (size_t)M - row_size ? lo[r] : (size_t)M - row_size;
		if (hi[r] == 0)
			left = 0;
		for (size_t j = 0; hi[r] && left + j < hi[r]; ++j)
			ctx->coef[(size_t)r * row_size + j] = (float)A_AT(left + j, r);
		ctx->offset[r] = (unsigned)left;
		ctx->lu_c[r] = (float)c[r];
		ctx->lu_l[r] = (float)(1.0 / (l[r] + eps));
		ctx->lu_u[r] = (float)u[r];
	}
#undef A_AT
	free(acol); free(aw); free(an); free(lo); free(hi);
	free(pl); free(pd); free(pu); free(c); free(l); free(u);
	return 0;
}

/* One horizontal pass (unresize_line_h_f32_c, unresize_impl.cpp:27-58) over h
 * lines, or one vertical pass (unresize_line_forward/back_v_f32_c,
 * unresize_impl.cpp:60-97) over w columns. Products and sums are rounded
 * one by one (no fused multiply-add). */
static void unresize_pass(const orc_unresize_ctx *x, int horizontal, unsigned w, unsigned h, const float *src,
                          ptrdiff_t ss, float *dst, ptrdiff_t ds)
{
	const ptrdiff_t sse = ss / 4, dse = ds / 4;
	if (horizontal) {
		for (unsigned i = 0; i < h; ++i) {
			const float *s = src + i * sse;
			float *d = dst + i * dse;
			float z = 0.0f, wv = 0.0f;
			for (unsigned j = 0; j < x->orig; ++j) {
				float accum = 0.0f;
				for (unsigned k = 0; k < x->row_size; ++k) {
					const float p = x->coef[(size_t)j * x->row_size + k] * s[x->offset[j] + k];
					accum = accum + p;
				}
				const float cz = x->lu_c[j] * z;
				z = (accum - cz) * x->lu_l[j];
				d[j] = z;
			}
			for (unsigned j = x->orig; j != 0; --j) {
				const float uw = x->lu_u[j - 1] * wv;
				wv = d[j - 1] - uw;
				d[j - 1] = wv;
			}
		}
	} else {
		for (unsigned j = 0; j < w; ++j) {
			float z = 0.0f;
			for (unsigned i = 0; i < x->orig; ++i) {
				float accum = 0.0f;
				for (unsigned k = 0; k < x->row_size; ++k) {
					const float p = x->coef[(size_t)i * x->row_size + k] * src[(x->offset[i] + k) * sse + j];
					accum = accum + p;
				}
				const float cz = x->lu_c[i] * z;
				z = (accum - cz) * x->lu_l[i];
				dst[i * dse + j] = z;
			}
			float wv = 0.0f;
			for (unsigned i = x->orig; i != 0; --i) {
				const float uw = x->lu_u[i - 1] * wv;
				wv = dst[(i - 1) * dse + j] - uw;
				dst[(i - 1) * dse + j] = wv;
			}
		}
	}
}

/* unresize_h_first (unresize.cpp:14-19) */
int orc_unresize_h_first(double xscale, double yscale)
{
	const double h = (xscale > 1.0 ? xscale : 1.0) * 2.0 + xscale * (yscale > 1.0 ? yscale : 1.0);
	const double v = (yscale > 1.0 ? yscale : 1.0) + yscale * (xscale > 1.0 ? xscale : 1.0) * 2.0;
	return h < v;
}

/* UnresizeConversion on one FLOAT plane (unresize.cpp:34-91): zero, one or
 * two passes; 0, or -2 for an upscale. */
int orc_unresize_plane(unsigned up_w, unsigned up_h, unsigned orig_w, unsigned orig_h, double shift_w,
                       double shift_h, const float *src, ptrdiff_t ss, float *dst, ptrdiff_t ds)
{
	const int skip_h = up_w == orig_w && shift_w == 0.0;
	const int skip_v = up_h == orig_h && shift_h == 0.0;
	if (orig_w > up_w || orig_h > up_h)
		return -2;
	if (skip_h && skip_v) {
		for (unsigned i = 0; i < up_h; ++i)
			memcpy((char *)dst + i * ds, (const char *)src + i * ss, (size_t)up_w * 4);
		return 0;
	}
	orc_unresize_ctx cw, ch;
	memset(&cw, 0, sizeof(cw));
	memset(&ch, 0, sizeof(ch));
	if (!skip_h && orc_unresize_context(orig_w, up_w, shift_w, &cw))
		return -2;
	if (!skip_v && orc_unresize_context(orig_h, up_h, shift_h, &ch)) {
		orc_unresize_ctx_free(&cw);
		return -2;
	}
	if (skip_h) {
		unresize_pass(&ch, 0, up_w, up_h, src, ss, dst, ds);
	} else if (skip_v) {
		unresize_pass(&cw, 1, up_w, up_h, src, ss, dst, ds);
	} else if (orc_unresize_h_first((double)orig_w / up_w, (double)orig_h / up_h)) {
		float *t = malloc(sizeof(float) * (size_t)orig_w * up_h);
		unresize_pass(&cw, 1, up_w, up_h, src, ss, t, (ptrdiff_t)orig_w * 4);
		unresize_pass(&ch, 0, orig_w, up_h, t, (ptrdiff_t)orig_w * 4, dst, ds);
		free(t);
	} else {
		float *t = malloc(sizeof(float) * (size_t)up_w * orig_h);
		unresize_pass(&ch, 0, up_w, up_h, src, ss, t, (ptrdiff_t)up_w * 4);
		unresize_pass(&cw, 1, up_w, orig_h, t, (ptrdiff_t)up_w * 4, dst, ds);
		free(t);
	}
	orc_unresize_ctx_free(&cw);
	orc_unresize_ctx_free(&ch);
	return 0;
}

/* ======================================================================
 * Colorspace conversion (src/zimg/colorspace/): zimg's ColorspaceConversion
 * on three FLOAT planes, C path (CPUClass::NONE). Enum values follow zimg's
 * internal order (colorspace.h:19-60), which fixes the order its path search
 * visits neighbours in.
 * ====================================================================== */

enum { CM_UNSPEC, CM_RGB, CM_601, CM_709, CM_FCC, CM_240M, CM_YCGCO, CM_2020_NCL, CM_2020_CL, CM_CHROM_NCL,
       CM_CHROM_CL, CM_LMS, CM_ICTCP, CM_COUNT };
enum { TC_UNSPEC, TC_LINEAR, TC_LOG100, TC_LOG316, TC_709, TC_470M, TC_470BG, TC_240M, TC_XVYCC, TC_1361, TC_SRGB,
       TC_2084, TC_428, TC_B67, TC_COUNT };
enum { CP_UNSPEC, CP_470M, CP_470BG, CP_SMPTE_C, CP_709, CP_FILM, CP_2020, CP_XYZ, CP_DCI_P3, CP_DCI_P3_D65,
       CP_EBU_3213_E, CP_COUNT };

typedef struct { int m, t, p; } orc_csp;
typedef struct { double v[3][3]; } orc_m3;
typedef struct { double v[3]; } orc_v3;

/* ---- transfer functions (gamma.cpp:12-343), float, libm ---- */
#define O_709_A 1.09929682680944f
#define O_709_B 0.018053968510807f
#define O_240_A 1.111572195921731f
#define O_240_B 0.022821585529445f
#define O_SRGB_A 1.055010718947587f
#define O_SRGB_B 0.003041282560128f
#define O_PQ_M1 0.1593017578125f
#define O_PQ_M2 78.84375f
#define O_PQ_C1 0.8359375f
#define O_PQ_C2 18.8515625f
#define O_PQ_C3 18.6875f
#define O_HLG_A 0.17883277f
#define O_HLG_B 0.28466892f
#define O_HLG_C 0.55991073f
#define O_PQ_OOTF 59.49080238715383f

/* fabs / copysign on the bits: gcc 13's floating-point range propagation
 * drops the fabsf inside copysignf(f(fabsf(x)), x) at -O2 when the call is
 * reached under x < 0 */
static float abs_bits(float x)
{
	uint32_t u;
	memcpy(&u, &x, 4);
	u &= 0x7FFFFFFFu;
	memcpy(&x, &u, 4);
	return x;
}
static float copysign_bits(float mag, float sgn)
{
	uint32_t a, b;
	memcpy(&a, &mag, 4);
	memcpy(&b, &sgn, 4);
	a = (a & 0x7FFFFFFFu) | (b & 0x80000000u);
	memcpy(&mag, &a, 4);
	return mag;
}
#define CSR float
#define CSN(n) n
#define CSPOW powf
#define CSLOG logf
#define CSLOG10 log10f
#define CSEXP expf
#define CSSQRT sqrtf
#define CSABS abs_bits
#define CSCOPYSIGN copysign_bits
#include "colorspace_tf.inc"
#undef CSR
#undef CSN
#undef CSPOW
#undef CSLOG
#undef CSLOG10
#undef CSEXP
#undef CSSQRT
#undef CSABS
#undef CSCOPYSIGN
#define CSR double
#define CSN(n) n##_d
#define CSPOW pow
#define CSLOG log
#define CSLOG10 log10
#define CSEXP exp
#define CSSQRT sqrt
#define CSABS fabs
#define CSCOPYSIGN copysign
#include "colorspace_tf.inc"
#undef CSR
#undef CSN
#undef CSPOW
#undef CSLOG
#undef CSLOG10
#undef CSEXP
#undef CSSQRT
#undef CSABS
#undef CSCOPYSIGN

typedef float (*orc_tf)(float);
typedef double (*orc_tfd)(double);
typedef struct {
	orc_tf to_linear, to_gamma;
	orc_tfd to_linear_d, to_gamma_d;  /* the same functions in FP64 */
	float to_linear_scale, to_gamma_scale;
} orc_transfer;

/* select_transfer_function (gamma.cpp:346-411) */
static orc_transfer orc_select_transfer(int t, double peak, int scene)
{
	orc_transfer f = { 0, 0, 0, 0, 1.0f, 1.0f };
	switch (t) {
	case TC_LOG100: f.to_linear = tlog100_i; f.to_linear_d = tlog100_i_d; f.to_gamma = tlog100; f.to_gamma_d = tlog100_d; break;
	case TC_LOG316: f.to_linear = tlog316_i; f.to_linear_d = tlog316_i_d; f.to_gamma = tlog316; f.to_gamma_d = tlog316_d; break;
	case TC_709: f.to_linear = scene ? t709_ioetf : t1886; f.to_linear_d = scene ? t709_ioetf_d : t1886_d; f.to_gamma = scene ? t709_oetf : t1886_i; f.to_gamma_d = scene ? t709_oetf_d : t1886_i_d; break;
	case TC_470M: f.to_linear = t470m; f.to_linear_d = t470m_d; f.to_gamma = t470m_i; f.to_gamma_d = t470m_i_d; break;
	case TC_470BG: f.to_linear = t470bg; f.to_linear_d = t470bg_d; f.to_gamma = t470bg_i; f.to_gamma_d = t470bg_i_d; break;
	case TC_240M: f.to_linear = scene ? t240_ioetf : t1886; f.to_linear_d = scene ? t240_ioetf_d : t1886_d; f.to_gamma = scene ? t240_oetf : t1886_i; f.to_gamma_d = scene ? t240_oetf_d : t1886_i_d; break;
	case TC_1361: f.to_linear = scene ? t1361_ioetf : t1361_eotf; f.to_linear_d = scene ? t1361_ioetf_d : t1361_eotf_d; f.to_gamma = scene ? t1361_oetf : t1361_ieotf; f.to_gamma_d = scene ? t1361_oetf_d : t1361_ieotf_d; break;
	case TC_XVYCC: f.to_linear = scene ? txvycc_ioetf : txvycc_eotf; f.to_linear_d = scene ? txvycc_ioetf_d : txvycc_eotf_d; f.to_gamma = scene ? txvycc_oetf : txvycc_ieotf; f.to_gamma_d = scene ? txvycc_oetf_d : txvycc_ieotf_d; break;
	case TC_SRGB: f.to_linear = tsrgb; f.to_linear_d = tsrgb_d; f.to_gamma = tsrgb_i; f.to_gamma_d = tsrgb_i_d; break;
	case TC_2084:
		f.to_linear = scene ? tpq_ioetf : tpq_eotf; f.to_linear_d = scene ? tpq_ioetf_d : tpq_eotf_d;
		f.to_gamma = scene ? tpq_oetf : tpq_ieotf; f.to_gamma_d = scene ? tpq_oetf_d : tpq_ieotf_d;
		f.to_linear_scale = (float)(10000.0f / peak);
		f.to_gamma_scale = (float)(peak / 10000.0f);
		break;
	case TC_428: f.to_linear = t428; f.to_linear_d = t428_d; f.to_gamma = t428_i; f.to_gamma_d = t428_i_d; break;
	case TC_B67:
		f.to_linear = scene ? thlg_ioetf : thlg_eotf; f.to_linear_d = scene ? thlg_ioetf_d : thlg_eotf_d;
		f.to_gamma = scene ? thlg_oetf : thlg_ieotf; f.to_gamma_d = scene ? thlg_oetf_d : thlg_ieotf_d;
		f.to_linear_scale = scene ? 12.0f : (float)(1000.0 / peak);
		f.to_gamma_scale = scene ? 1.0f / 12.0f : (float)(peak / 1000.0);
		break;
	default: break;
	}
	return f;
}

/* ---- 3x3 algebra in double (matrix3.cpp) ---- */
static orc_m3 m3_mul(orc_m3 a, orc_m3 b)
{
	orc_m3 r;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) {
			double acc = 0;
			for (int k = 0; k < 3; ++k)
				acc += a.v[i][k] * b.v[k][j];
			r.v[i][j] = acc;
		}
	return r;
}
static orc_v3 m3_apply(orc_m3 m, orc_v3 x)
{
	orc_v3 r;
	for (int i = 0; i < 3; ++i) {
		double acc = 0;
		for (int k = 0; k < 3; ++k)
			acc += m.v[i][k] * x.v[k];
		r.v[i] = acc;
	}
	return r;
}
static double det2(double a, double b, double c, double d) { return a * d - b * c; }
static orc_m3 m3_inverse(orc_m3 m)
{
	const double (*a)[3] = m.v;
	double det = 0;
	det += a[0][0] * det2(a[1][1], a[1][2], a[2][1], a[2][2]);
	det -= a[0][1] * det2(a[1][0], a[1][2], a[2][0], a[2][2]);
	det += a[0][2] * det2(a[1][0], a[1][1], a[2][0], a[2][1]);
	orc_m3 r;
	r.v[0][0] = det2(a[1][1], a[1][2], a[2][1], a[2][2]) / det;
	r.v[0][1] = det2(a[0][2], a[0][1], a[2][2], a[2][1]) / det;
	r.v[0][2] = det2(a[0][1], a[0][2], a[1][1], a[1][2]) / det;
	r.v[1][0] = det2(a[1][2], a[1][0], a[2][2], a[2][0]) / det;
	r.v[1][1] = det2(a[0][0], a[0][2], a[2][0], a[2][2]) / det;
	r.v[1][2] = det2(a[0][2], a[0][0], a[1][2], a[1][0]) / det;
	r.v[2][0] = det2(a[1][0], a[1][1], a[2][0], a[2][1]) / det;
	r.v[2][1] = det2(a[0][1], a[0][0], a[2][1], a[2][0]) / det;
	r.v[2][2] = det2(a[0][0], a[0][1], a[1][0], a[1][1]) / det;
	return r;
}
static orc_m3 m3_identity(void)
{
	orc_m3 r = { { { 1, 0, 0 }, { 0, 1, 0 }, { 0, 0, 1 } } };
	return r;
}
static orc_v3 xy_to_xyz(double x, double y)
{
	orc_v3 r = { { x / y, 1.0, (1.0 - x - y) / y } };
	return r;
}
static orc_v3 v3_cross(orc_v3 a, orc_v3 b)
{
	orc_v3 r = { { a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2], a.v[0] * b.v[1] - a.v[1] * b.v[0] } };
	return r;
}
static double v3_dot(orc_v3 a, orc_v3 b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]; }

/* ---- colorimetry (colorspace_param.cpp/.h): published constants ---- */
static void yuv_kr_kb(int m, double *kr, double *kb)
{
	switch (m) {
	case CM_FCC: *kr = 0.3; *kb = 0.11; break;
	case CM_240M: *kr = 0.212; *kb = 0.087; break;
	case CM_601: *kr = 0.299; *kb = 0.114; break;
	case CM_709: *kr = 0.2126; *kb = 0.0722; break;
	case CM_2020_NCL: case CM_2020_CL: *kr = 0.2627; *kb = 0.0593; break;
	default: *kr = 0; *kb = 0; break;
	}
}
static orc_v3 white_point(int p)
{
	switch (p) {
	case CP_470M: case CP_FILM: return xy_to_xyz(0.31, 0.316);                 /* illuminant C */
	case CP_XYZ: return xy_to_xyz(1.0 / 3.0, 1.0 / 3.0);                        /* illuminant E */
	case CP_DCI_P3: return xy_to_xyz(0.314, 0.351);                             /* DCI white */
	default: return xy_to_xyz(0.3127, 0.3290);                                  /* D65 */
	}
}
static void primaries_xy(int p, double o[3][2])
{
	static const double t470m[3][2] = { { 0.670, 0.330 }, { 0.210, 0.710 }, { 0.140, 0.080 } };
	static const double t470bg[3][2] = { { 0.640, 0.330 }, { 0.290, 0.600 }, { 0.150, 0.060 } };
	static const double smptec[3][2] = { { 0.630, 0.340 }, { 0.310, 0.595 }, { 0.155, 0.070 } };
	static const double r709[3][2] = { { 0.640, 0.330 }, { 0.300, 0.600 }, { 0.150, 0.060 } };
	static const double film[3][2] = { { 0.681, 0.319 }, { 0.243, 0.692 }, { 0.145, 0.049 } };
	static const double r2020[3][2] = { { 0.708, 0.292 }, { 0.170, 0.797 }, { 0.131, 0.046 } };
	static const double p3[3][2] = { { 0.680, 0.320 }, { 0.265, 0.690 }, { 0.150, 0.060 } };
	static const double ebu[3][2] = { { 0.630, 0.340 }, { 0.295, 0.605 }, { 0.155, 0.077 } };
	const double (*s)[2] = r709;
	switch (p) {
	case CP_470M: s = t470m; break;
	case CP_470BG: s = t470bg; break;
	case CP_SMPTE_C: s = smptec; break;
	case CP_FILM: s = film; break;
	case CP_2020: s = r2020; break;
	case CP_DCI_P3: case CP_DCI_P3_D65: s = p3; break;
	case CP_EBU_3213_E: s = ebu; break;
	default: break;
	}
	memcpy(o, s, sizeof(r709));
}
static orc_m3 rgb_to_yuv_kr_kb(double kr, double kb)
{
	const double kg = 1.0 - kr - kb, us = 1.0 / (2.0 - 2.0 * kb), vs = 1.0 / (2.0 - 2.0 * kr);
	orc_m3 r = { { { kr, kg, kb }, { -kr * us, -kg * us, (1.0 - kb) * us }, { (1.0 - kr) * vs, -kg * vs, -kb * vs } } };
	return r;
}
static orc_m3 ncl_rgb_to_yuv(int m)
{
	if (m == CM_YCGCO) {
		orc_m3 r = { { { 0.25, 0.5, 0.25 }, { -0.25, 0.5, -0.25 }, { 0.5, 0, -0.5 } } };
		return r;
	}
	if (m == CM_LMS) {
		orc_m3 r = { { { 1688.0 / 4096.0, 2146.0 / 4096.0, 262.0 / 4096.0 },
		               { 683.0 / 4096.0, 2951.0 / 4096.0, 462.0 / 4096.0 },
		               { 99.0 / 4096.0, 309.0 / 4096.0, 3688.0 / 4096.0 } } };
		return r;
	}
	double kr, kb;
	yuv_kr_kb(m, &kr, &kb);
	return rgb_to_yuv_kr_kb(kr, kb);
}
/* ITU-T H.273 E-22..E-27 */
static void kr_kb_from_primaries(int p, double *kr, double *kb)
{
	double xy[3][2];
	primaries_xy(p, xy);
	const orc_v3 r = xy_to_xyz(xy[0][0], xy[0][1]), g = xy_to_xyz(xy[1][0], xy[1][1]), b = xy_to_xyz(xy[2][0], xy[2][1]);
	const orc_v3 w = white_point(p);
	const orc_v3 xr = { { r.v[0], g.v[0], b.v[0] } }, yr = { { r.v[1], g.v[1], b.v[1] } }, zr = { { r.v[2], g.v[2], b.v[2] } };
	const double den = v3_dot(xr, v3_cross(yr, zr));
	*kr = v3_dot(w, v3_cross(g, b)) / den;
	*kb = v3_dot(w, v3_cross(r, g)) / den;
}
static orc_m3 ncl_rgb_to_yuv_from_primaries(int p)
{
	if (p == CP_709)
		return ncl_rgb_to_yuv(CM_709);
	if (p == CP_2020)
		return ncl_rgb_to_yuv(CM_2020_NCL);
	double kr, kb;
	kr_kb_from_primaries(p, &kr, &kb);
	return rgb_to_yuv_kr_kb(kr, kb);
}
static orc_m3 lms_to_ictcp(int t)
{
	if (t == TC_B67) {
		orc_m3 r = { { { 0.5, 0.5, 0.0 }, { 3625.0 / 4096.0, -7465.0 / 4096.0, 3840.0 / 4096.0 },
		               { 9500.0 / 4096.0, -9212.0 / 4096.0, -288.0 / 4096.0 } } };
		return r;
	}
	orc_m3 r = { { { 0.5, 0.5, 0.0 }, { 6610.0 / 4096.0, -13613.0 / 4096.0, 7003.0 / 4096.0 },
	               { 17933.0 / 4096.0, -17390.0 / 4096.0, -543.0 / 4096.0 } } };
	return r;
}
static orc_m3 rgb_to_xyz(int p)
{
	if (p == CP_XYZ)
		return m3_identity();
	double xy[3][2];
	primaries_xy(p, xy);
	orc_m3 cols;  /* rows X, Y, Z; columns R, G, B */
	for (int c = 0; c < 3; ++c) {
		const orc_v3 v = xy_to_xyz(xy[c][0], xy[c][1]);
		for (int r = 0; r < 3; ++r)
			cols.v[r][c] = v.v[r];
	}
	const orc_v3 s = m3_apply(m3_inverse(cols), white_point(p));
	orc_m3 m;
	for (int r = 0; r < 3; ++r)
		for (int c = 0; c < 3; ++c)
			m.v[r][c] = cols.v[r][c] * s.v[c];
	return m;
}
static orc_m3 xyz_to_rgb(int p)
{
	if (p == CP_XYZ)
		return m3_identity();
	return m3_inverse(rgb_to_xyz(p));
}
/* Bradford adaptation (http://www.brucelindbloom.com, Eqn_ChromAdapt) */
static orc_m3 white_adapt(int in, int out)
{
	const orc_m3 br = { { { 0.8951, 0.2664, -0.1614 }, { -0.7502, 1.7135, 0.0367 }, { 0.0389, -0.0685, 1.0296 } } };
	const orc_v3 wi = white_point(in), wo = white_point(out);
	if (wi.v[0] == wo.v[0] && wi.v[1] == wo.v[1] && wi.v[2] == wo.v[2])
		return m3_identity();
	const orc_v3 ri = m3_apply(br, wi), ro = m3_apply(br, wo);
	orc_m3 d = { { { 0 } } };
	for (int k = 0; k < 3; ++k)
		d.v[k][k] = ro.v[k] / ri.v[k];
	return m3_mul(m3_mul(m3_inverse(br), d), br);
}

/* ---- the path between two colorspaces (colorspace_graph.cpp) ---- */
enum { E_NCL_YUV2RGB, E_NCL_RGB2YUV, E_ICTCP2LMS, E_LMS2ICTCP, E_G2L, E_L2G, E_CL_YUV2RGB, E_CL_RGB2YUV, E_GAMUT };

static int csp_key(orc_csp c) { return (c.m * TC_COUNT + c.t) * CP_COUNT + c.p; }
static int csp_eq(orc_csp a, orc_csp b) { return a.m == b.m && a.t == b.t && a.p == b.p; }

static int csp_valid(orc_csp c)
{
	if (c.m == CM_2020_CL && c.t != TC_709)
		return 0;
	if ((c.m == CM_CHROM_NCL || c.m == CM_CHROM_CL) && c.p == CP_UNSPEC)
		return 0;
	if (c.m == CM_ICTCP && !((c.t == TC_2084 || c.t == TC_B67) && c.p == CP_2020))
		return 0;
	if (c.m == CM_LMS && !((c.t == TC_LINEAR || c.t == TC_2084 || c.t == TC_B67) && c.p == CP_2020))
		return 0;
	return 1;
}

typedef struct { orc_csp to; int edge; } orc_edge;

static int neighbours(orc_csp c, orc_edge *e)
{
	int n = 0;
#define ADD(M, T, P, E) do { e[n].to.m = (M); e[n].to.t = (T); e[n].to.p = (P); e[n].edge = (E); ++n; } while (0)
	if (c.m == CM_RGB) {
		for (int m = 0; m < CM_COUNT; ++m) {
			if (m == CM_UNSPEC || m == CM_RGB || m == CM_2020_CL || m == CM_CHROM_NCL || m == CM_CHROM_CL || m == CM_LMS ||
			    m == CM_ICTCP)
				continue;
			ADD(m, c.t, c.p, E_NCL_RGB2YUV);
		}
		if (c.p != CP_UNSPEC)
			ADD(CM_CHROM_NCL, c.t, c.p, E_NCL_RGB2YUV);
		if (c.t == TC_LINEAR) {
			for (int t = 0; t < TC_COUNT; ++t) {
				if (t == c.t || t == TC_UNSPEC)
					continue;
				ADD(c.m, t, c.p, E_L2G);
				if (c.p != CP_UNSPEC)
					ADD(CM_CHROM_CL, t, c.p, E_CL_RGB2YUV);
			}
			if (c.p != CP_UNSPEC)
				for (int p = 0; p < CP_COUNT; ++p)
					if (p != c.p && p != CP_UNSPEC)
						ADD(c.m, c.t, p, E_GAMUT);
			ADD(CM_2020_CL, TC_709, c.p, E_CL_RGB2YUV);
			if (c.p == CP_2020)
				ADD(CM_LMS, c.t, c.p, E_NCL_RGB2YUV);
		} else if (c.t != TC_UNSPEC) {
			ADD(c.m, TC_LINEAR, c.p, E_G2L);
		}
	} else if (c.m == CM_2020_CL || c.m == CM_CHROM_CL) {
		ADD(CM_RGB, TC_LINEAR, c.p, E_CL_YUV2RGB);
	} else if (c.m == CM_LMS) {
		if (c.t == TC_2084 || c.t == TC_B67) {
			ADD(CM_ICTCP, c.t, c.p, E_LMS2ICTCP);
			ADD(c.m, TC_LINEAR, c.p, E_G2L);
		}
		if (c.t == TC_LINEAR) {
			ADD(CM_RGB, c.t, c.p, E_NCL_YUV2RGB);
			ADD(c.m, TC_2084, c.p, E_L2G);
			ADD(c.m, TC_B67, c.p, E_L2G);
		}
	} else if (c.m == CM_ICTCP) {
		if (c.t == TC_2084 || c.t == TC_B67)
			ADD(CM_LMS, c.t, c.p, E_ICTCP2LMS);
	} else if (c.m != CM_UNSPEC) {
		ADD(CM_RGB, c.t, c.p, E_NCL_YUV2RGB);
	}
#undef ADD
	return n;
}

/* Breadth-first search from in to out; returns the number of edges (at most
 * 6 used by zimg) written to steps[]/froms[], or -1 if there is no path. */
static int csp_path(orc_csp in, orc_csp out, int *edges, orc_csp *froms, int max)
{
	enum { NKEY = CM_COUNT * TC_COUNT * CP_COUNT };
	char *visited = calloc(NKEY, 1);
	int *parent = malloc(sizeof(int) * NKEY), *pedge = malloc(sizeof(int) * NKEY);
	orc_csp *queue = malloc(sizeof(orc_csp) * NKEY);
	int head = 0, tail = 0, found = 0;
	orc_csp v = in;
	visited[csp_key(in)] = 1;
	queue[tail++] = in;
	while (head < tail) {
		v = queue[head++];
		if (csp_eq(v, out)) {
			found = 1;
			break;
		}
		orc_edge e[64];
		const int n = neighbours(v, e);
		for (int k = 0; k < n; ++k) {
			const int key = csp_key(e[k].to);
			if (visited[key])
				continue;
			visited[key] = 1;
			queue[tail++] = e[k].to;
			parent[key] = csp_key(v);
			pedge[key] = e[k].edge;
		}
	}
	int len = -1;
	if (found) {
		int rev_e[64], rev_k[64], cnt = 0, key = csp_key(out);
		while (key != csp_key(in) && cnt < 64) {
			rev_e[cnt] = pedge[key];
			rev_k[cnt] = parent[key];
			key = parent[key];
			++cnt;
		}
		if (cnt <= max) {
			for (int k = 0; k < cnt; ++k) {
				edges[k] = rev_e[cnt - 1 - k];
				const int fk = rev_k[cnt - 1 - k];
				froms[k].p = fk % CP_COUNT;
				froms[k].t = (fk / CP_COUNT) % TC_COUNT;
				froms[k].m = fk / (CP_COUNT * TC_COUNT);
			}
			len = cnt;
		}
	}
	free(visited);
	free(parent);
	free(pedge);
	free(queue);
	return len;
}

/* ---- operations (operation.cpp, operation_impl.cpp C classes) ---- */
enum { OP_MATRIX, OP_GAMMA, OP_HLG, OP_HLG_INV, OP_CL2RGB, OP_CL2YUV };
typedef struct {
	int kind;
	float m[3][3];
	orc_tf f, g;       /* GAMMA: f; CL2RGB: f to linear; CL2YUV: f to gamma */
	orc_tfd fd;        /* f in FP64 */
	float pre, post;   /* GAMMA */
	float kr, kg, kb, scale, nb, pb, nr, pr;
} orc_op;

struct orc_colorspace {
	int nops;
	orc_op ops[6];
};

static orc_op op_matrix(orc_m3 m)
{
	orc_op o;
	memset(&o, 0, sizeof(o));
	o.kind = OP_MATRIX;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			o.m[i][j] = (float)m.v[i][j];
	return o;
}

static orc_op make_op(int edge, orc_csp in, orc_csp out, double peak, int approx, int scene, int adapt)
{
	orc_op o;
	memset(&o, 0, sizeof(o));
	const int b67_display_in = in.p != CP_UNSPEC && !approx && !scene;
	const int b67_display_out = out.p != CP_UNSPEC && !approx && !scene;
	switch (edge) {
	case E_NCL_YUV2RGB:
		return op_matrix(m3_inverse(in.m == CM_CHROM_NCL ? ncl_rgb_to_yuv_from_primaries(in.p) : ncl_rgb_to_yuv(in.m)));
	case E_NCL_RGB2YUV:
		return op_matrix(out.m == CM_CHROM_NCL ? ncl_rgb_to_yuv_from_primaries(out.p) : ncl_rgb_to_yuv(out.m));
	case E_ICTCP2LMS: return op_matrix(m3_inverse(lms_to_ictcp(in.t)));
	case E_LMS2ICTCP: return op_matrix(lms_to_ictcp(in.t));
	case E_G2L:
		if (in.t == TC_B67 && b67_display_in) {
			const orc_m3 m = ncl_rgb_to_yuv_from_primaries(in.p);
			o.kind = OP_HLG_INV;
			o.kr = (float)m.v[0][0]; o.kg = (float)m.v[0][1]; o.kb = (float)m.v[0][2];
			o.scale = orc_select_transfer(TC_B67, peak, 0).to_linear_scale;
		} else {
			const orc_transfer f = orc_select_transfer(in.t, peak, scene);
			o.kind = OP_GAMMA; o.f = f.to_linear; o.fd = f.to_linear_d; o.pre = 1.0f; o.post = f.to_linear_scale;
		}
		return o;
	case E_L2G:
		if (out.t == TC_B67 && b67_display_out) {
			const orc_m3 m = ncl_rgb_to_yuv_from_primaries(out.p);
			o.kind = OP_HLG;
			o.kr = (float)m.v[0][0]; o.kg = (float)m.v[0][1]; o.kb = (float)m.v[0][2];
			o.scale = orc_select_transfer(TC_B67, peak, 0).to_gamma_scale;
		} else {
			const orc_transfer f = orc_select_transfer(out.t, peak, scene);
			o.kind = OP_GAMMA; o.f = f.to_gamma; o.fd = f.to_gamma_d; o.pre = f.to_gamma_scale; o.post = 1.0f;
		}
		return o;
	case E_GAMUT: {
		orc_m3 m = adapt ? m3_mul(m3_mul(xyz_to_rgb(out.p), white_adapt(in.p, out.p)), rgb_to_xyz(in.p))
		                 : m3_mul(xyz_to_rgb(out.p), rgb_to_xyz(in.p));
		return op_matrix(m);
	}
	case E_CL_YUV2RGB: {
		const orc_transfer f = orc_select_transfer(in.t, peak, 1);
		const orc_m3 m = in.m == CM_CHROM_CL ? ncl_rgb_to_yuv_from_primaries(in.p) : ncl_rgb_to_yuv(in.m);
		o.kind = OP_CL2RGB; o.f = f.to_linear; o.fd = f.to_linear_d; o.g = f.to_gamma;
		o.kr = (float)m.v[0][0]; o.kg = (float)m.v[0][1]; o.kb = (float)m.v[0][2];
		o.scale = f.to_linear_scale;
		o.nb = f.to_gamma(1.0f - (float)m.v[0][2]);
		o.pb = 1.0f - f.to_gamma((float)m.v[0][2]);
		o.nr = f.to_gamma(1.0f - (float)m.v[0][0]);
		o.pr = 1.0f - f.to_gamma((float)m.v[0][0]);
		return o;
	}
	case E_CL_RGB2YUV: {
		const orc_transfer f = orc_select_transfer(out.t, peak, 1);
		const orc_m3 m = out.m == CM_CHROM_CL ? ncl_rgb_to_yuv_from_primaries(out.p) : ncl_rgb_to_yuv(out.m);
		o.kind = OP_CL2YUV; o.f = f.to_gamma; o.fd = f.to_gamma_d;
		o.kr = (float)m.v[0][0]; o.kg = (float)m.v[0][1]; o.kb = (float)m.v[0][2];
		o.scale = f.to_gamma_scale;
		o.nb = f.to_gamma(1.0f - (float)m.v[0][2]);
		o.pb = 1.0f - f.to_gamma((float)m.v[0][2]);
		o.nr = f.to_gamma(1.0f - (float)m.v[0][0]);
		o.pr = 1.0f - f.to_gamma((float)m.v[0][0]);
		return o;
	}
	default: return o;
	}
}

/* ColorspaceConversion::create (colorspace.cpp:94-121): SMPTE 240M transfer
 * read as BT.709 unless scene-referred; no operations when the effective
 * colorspaces are equal. Arguments are zimg's internal enum values. Returns
 * NULL with *err set (-1 invalid colorspace or no path, -2 no memory). */
struct orc_colorspace *orc_colorspace_create(int m_in, int t_in, int p_in, int m_out, int t_out, int p_out,
                                             double peak, int approx, int scene, int adapt, int *err)
{
	*err = 0;
	orc_csp in = { m_in, t_in, p_in }, out = { m_out, t_out, p_out };
	if (!scene) {
		if (in.t == TC_240M)
			in.t = TC_709;
		if (out.t == TC_240M)
			out.t = TC_709;
	}
	struct orc_colorspace *c = calloc(1, sizeof(*c));
	if (!c) {
		*err = -2;
		return NULL;
	}
	if (csp_eq(in, out))
		return c;
	if (!csp_valid(in) || !csp_valid(out)) {
		free(c);
		*err = -1;
		return NULL;
	}
	int edges[6];
	orc_csp froms[6];
	const int n = csp_path(in, out, edges, froms, 6);
	if (n < 0) {
		free(c);
		*err = -1;
		return NULL;
	}
	for (int k = 0; k < n; ++k) {
		const orc_csp to = k + 1 < n ? froms[k + 1] : out;
		c->ops[k] = make_op(edges[k], froms[k], to, peak, approx, scene, adapt);
	}
	c->nops = n;
	return c;
}

void orc_colorspace_free(struct orc_colorspace *c)
{
	free(c);
}

int orc_colorspace_num_ops(const struct orc_colorspace *c)
{
	return c->nops;
}

/* Kind of operation k (OP_* order: matrix, gamma, HLG, inverse HLG, CL to
 * RGB, CL to YUV), and its float matrix when it has one. */
int orc_colorspace_op(const struct orc_colorspace *c, int k, float *m9)
{
	if (k < 0 || k >= c->nops)
		return -1;
	if (m9)
		memcpy(m9, c->ops[k].m, sizeof(c->ops[k].m));
	return c->ops[k].kind;
}

static void apply_op(const orc_op *o, float *a, float *b, float *c)
{
	switch (o->kind) {
	case OP_MATRIX: {
		const float x = o->m[0][0] * *a + o->m[0][1] * *b + o->m[0][2] * *c;
		const float y = o->m[1][0] * *a + o->m[1][1] * *b + o->m[1][2] * *c;
		const float z = o->m[2][0] * *a + o->m[2][1] * *b + o->m[2][2] * *c;
		*a = x; *b = y; *c = z;
		break;
	}
	case OP_GAMMA:
		*a = o->post * o->f(*a * o->pre);
		*b = o->post * o->f(*b * o->pre);
		*c = o->post * o->f(*c * o->pre);
		break;
	case OP_HLG: {
		const float gamma = 1.2f;
		float r = *a * o->scale, g = *b * o->scale, bb = *c * o->scale;
		float yd = o->kr * r + o->kg * g + o->kb * bb;
		yd = yd < FLT_MIN ? FLT_MIN : yd;
		const float ys_inv = powf(yd, (1.0f - gamma) / gamma);
		*a = thlg_oetf(r * ys_inv);
		*b = thlg_oetf(g * ys_inv);
		*c = thlg_oetf(bb * ys_inv);
		break;
	}
	case OP_HLG_INV: {
		const float gamma = 1.2f;
		float r = thlg_ioetf(*a), g = thlg_ioetf(*b), bb = thlg_ioetf(*c);
		float ys = o->kr * r + o->kg * g + o->kb * bb;
		ys = ys < FLT_MIN ? FLT_MIN : ys;
		ys = powf(ys, gamma - 1.0f);
		r = r * ys; g = g * ys; bb = bb * ys;
		*a = r * o->scale; *b = g * o->scale; *c = bb * o->scale;
		break;
	}
	case OP_CL2RGB: {
		const float y = *a, u = *b, v = *c;
		const float bmy = u < 0 ? u * 2.0f * o->nb : u * 2.0f * o->pb;
		const float rmy = v < 0 ? v * 2.0f * o->nr : v * 2.0f * o->pr;
		const float bb = o->f(bmy + y), r = o->f(rmy + y), yl = o->f(y);
		const float g = (yl - o->kr * r - o->kb * bb) / o->kg;
		*a = r * o->scale; *b = g * o->scale; *c = bb * o->scale;
		break;
	}
	case OP_CL2YUV: {
		float r = *a * o->scale, g = *b * o->scale, bb = *c * o->scale;
		const float y = o->f(o->kr * r + o->kg * g + o->kb * bb);
		bb = o->f(bb);
		r = o->f(r);
		const float u = (bb - y < 0.0f) ? (bb - y) / (2.0f * o->nb) : (bb - y) / (2.0f * o->pb);
		const float v = (r - y < 0.0f) ? (r - y) / (2.0f * o->nr) : (r - y) / (2.0f * o->pr);
		*a = y; *b = u; *c = v;
		break;
	}
	default: break;
	}
}

/* The same operation in FP64 with the same float parameters: the error of
 * a float evaluation is measured against this. */
static void apply_op_d(const orc_op *o, double *a, double *b, double *c)
{
	switch (o->kind) {
	case OP_MATRIX: {
		const double x = (double)o->m[0][0] * *a + (double)o->m[0][1] * *b + (double)o->m[0][2] * *c;
		const double y = (double)o->m[1][0] * *a + (double)o->m[1][1] * *b + (double)o->m[1][2] * *c;
		const double z = (double)o->m[2][0] * *a + (double)o->m[2][1] * *b + (double)o->m[2][2] * *c;
		*a = x; *b = y; *c = z;
		break;
	}
	case OP_GAMMA:
		*a = o->post * o->fd(*a * o->pre);
		*b = o->post * o->fd(*b * o->pre);
		*c = o->post * o->fd(*c * o->pre);
		break;
	case OP_HLG: {
		const double gamma = 1.2f;
		double r = *a * o->scale, g = *b * o->scale, bb = *c * o->scale;
		double yd = o->kr * r + o->kg * g + o->kb * bb;
		yd = yd < FLT_MIN ? FLT_MIN : yd;
		const double ys_inv = pow(yd, (double)((1.0f - 1.2f) / 1.2f));
		(void)gamma;
		*a = thlg_oetf_d(r * ys_inv);
		*b = thlg_oetf_d(g * ys_inv);
		*c = thlg_oetf_d(bb * ys_inv);
		break;
	}
	case OP_HLG_INV: {
		double r = thlg_ioetf_d(*a), g = thlg_ioetf_d(*b), bb = thlg_ioetf_d(*c);
		double ys = o->kr * r + o->kg * g + o->kb * bb;
		ys = ys < FLT_MIN ? FLT_MIN : ys;
		ys = pow(ys, (double)(1.2f - 1.0f));
		*a = r * ys * o->scale; *b = g * ys * o->scale; *c = bb * ys * o->scale;
		break;
	}
	case OP_CL2RGB: {
		const double y = *a, u = *b, v = *c;
		const double bmy = u < 0 ? u * 2.0 * o->nb : u * 2.0 * o->pb;
		const double rmy = v < 0 ? v * 2.0 * o->nr : v * 2.0 * o->pr;
		const double bb = o->fd(bmy + y), r = o->fd(rmy + y), yl = o->fd(y);
		const double g = (yl - o->kr * r - o->kb * bb) / o->kg;
		*a = r * o->scale; *b = g * o->scale; *c = bb * o->scale;
		break;
	}
	case OP_CL2YUV: {
		double r = *a * o->scale, g = *b * o->scale, bb = *c * o->scale;
		const double y = o->fd(o->kr * r + o->kg * g + o->kb * bb);
		bb = o->fd(bb);
		r = o->fd(r);
		*a = y;
		*b = (bb - y < 0.0) ? (bb - y) / (2.0 * o->nb) : (bb - y) / (2.0 * o->pb);
		*c = (r - y < 0.0) ? (r - y) / (2.0 * o->nr) : (r - y) / (2.0 * o->pr);
		break;
	}
	default: break;
	}
}

/* Three FLOAT planes through the conversion evaluated in FP64, into three
 * double planes (strides in bytes). */
void orc_colorspace_run_f64(const struct orc_colorspace *c, unsigned w, unsigned h, const void *const src[3],
                            const ptrdiff_t src_stride[3], void *const dst[3], const ptrdiff_t dst_stride[3])
{
	for (unsigned i = 0; i < h; ++i) {
		for (unsigned j = 0; j < w; ++j) {
			double v[3];
			for (int p = 0; p < 3; ++p)
				v[p] = ((const float *)((const char *)src[p] + (ptrdiff_t)i * src_stride[p]))[j];
			for (int k = 0; k < c->nops; ++k)
				apply_op_d(&c->ops[k], &v[0], &v[1], &v[2]);
			for (int p = 0; p < 3; ++p)
				((double *)((char *)dst[p] + (ptrdiff_t)i * dst_stride[p]))[j] = v[p];
		}
	}
}

/* Three FLOAT planes (strides in bytes) through the conversion. */
void orc_colorspace_run(const struct orc_colorspace *c, unsigned w, unsigned h, const void *const src[3],
                        const ptrdiff_t src_stride[3], void *const dst[3], const ptrdiff_t dst_stride[3])
{
	for (unsigned i = 0; i < h; ++i) {
		const float *s0 = (const float *)((const char *)src[0] + (ptrdiff_t)i * src_stride[0]);
		const float *s1 = (const float *)((const char *)src[1] + (ptrdiff_t)i * src_stride[1]);
		const float *s2 = (const float *)((const char *)src[2] + (ptrdiff_t)i * src_stride[2]);
		float *d0 = (float *)((char *)dst[0] + (ptrdiff_t)i * dst_stride[0]);
		float *d1 = (float *)((char *)dst[1] + (ptrdiff_t)i * dst_stride[1]);
		float *d2 = (float *)((char *)dst[2] + (ptrdiff_t)i * dst_stride[2]);
		for (unsigned j = 0; j < w; ++j) {
			float a = s0[j], b = s1[j], cc = s2[j];
			for (int k = 0; k < c->nops; ++k)
				apply_op(&c->ops[k], &a, &b, &cc);
			d0[j] = a;
			d1[j] = b;
			d2[j] = cc;
		}
	}
}
