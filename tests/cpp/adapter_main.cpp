// Drives zg::GraphengineResizePass the way a graph drives a filter: build it
// from pass parameters, read its descriptor, call process() for every output
// line in steps of descriptor().step. Reads a raw u16 plane, writes the
// resized plane. Usage: adapter_main in.raw w h horizontal dst_dim depth out.raw
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>

#include "graphengine/filter.h"
#include "zimg_gb300_filter.hpp"

using Pass = zg::GraphengineResizePass<graphengine::Filter, graphengine::BufferDescriptor, graphengine::FilterDescriptor>;

int main(int argc, char **argv)
{
	if (argc != 8)
		return 2;
	const unsigned w = std::atoi(argv[2]), h = std::atoi(argv[3]);
	zg_pass_params p{};
	p.src_width = w;
	p.src_height = h;
	p.pixel_type = ZG_PIXEL_WORD;
	p.depth = std::atoi(argv[6]);
	p.horizontal = std::atoi(argv[4]);
	p.dst_dim = std::atoi(argv[5]);
	p.filter = ZG_RESIZE_SPLINE36;
	p.filter_param_a = p.filter_param_b = 0.0 / 0.0;
	p.shift = 0.0;
	p.subwidth = 0.0 / 0.0;

	std::vector<unsigned short> src(static_cast<size_t>(w) * h);
	FILE *f = std::fopen(argv[1], "rb");
	if (!f || std::fread(src.data(), 2, src.size(), f) != src.size())
		return 3;
	std::fclose(f);

	try {
		Pass pass(p);
		const graphengine::FilterDescriptor &d = pass.descriptor();
		const unsigned ow = d.format.width, oh = d.format.height;
		void *din = nullptr, *dout = nullptr;
		if (cudaMalloc(&din, src.size() * 2) || cudaMalloc(&dout, static_cast<size_t>(ow) * oh * 2))
			return 4;
		cudaMemcpy(din, src.data(), src.size() * 2, cudaMemcpyHostToDevice);
		const graphengine::BufferDescriptor in{ din, static_cast<std::ptrdiff_t>(w) * 2, ZG_BUFFER_MAX };
		const graphengine::BufferDescriptor out{ dout, static_cast<std::ptrdiff_t>(ow) * 2, ZG_BUFFER_MAX };
		pass.init_context(nullptr);
		for (unsigned i = 0; i < oh; i += d.step)
			pass.process(&in, &out, i, 0, ow, nullptr, nullptr);
		if (pass.status() != ZG_ERROR_SUCCESS || cudaDeviceSynchronize() != cudaSuccess)
			return 5;
		std::vector<unsigned short> dst(static_cast<size_t>(ow) * oh);
		cudaMemcpy(dst.data(), dout, dst.size() * 2, cudaMemcpyDeviceToHost);
		f = std::fopen(argv[7], "wb");
		std::fwrite(dst.data(), 2, dst.size(), f);
		std::fclose(f);
		std::printf("%u %u %u %u %u\n", ow, oh, d.step, pass.get_row_deps(0).second, pass.get_col_deps(0, 1).second);
		cudaFree(din);
		cudaFree(dout);
	} catch (const zg::Exception &e) {
		std::fprintf(stderr, "zg error %d: %s\n", e.code, e.what());
		return 6;
	}
	return 0;
}
