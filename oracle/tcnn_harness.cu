// TEST INFRASTRUCTURE ONLY -- never linked into libnlod.so.
//
// A small C ABI over tiny-cuda-nn, compiled from the reference's vendored sources
// (rptr/ext/tiny-cuda-nn, staged and built by oracle/build_tcnn.py into oracle/_ref/).  It lets
// the parity tests, the golden-vector script and the bench's comparison leg drive the reference
// network path on the same GPU, with weights injected from the same FP32 vector:
//
//   tch_create           tcnn::create_from_config (include/tiny-cuda-nn/config.h:51-62): a
//                        NetworkWithInputEncoding<__half> + Trainer<float,__half,__half> + loss +
//                        optimizer, exactly the objects neural_lod builds
//                        (rptr/cuda/neural-lod/neural_lod_learning_init.cu:654-668)
//   tch_set_params       Trainer::set_params_full_precision (trainer.h:234-246), network then
//                        encoding, as NetworkWithInputEncoding lays them out (:113-128)
//   tch_set_max_level_gpu  GridEncoding::set_max_level_gpu (encodings/grid.h:918-920) on the grid
//                        nested inside the composite
//   tch_inference        Network::inference (object.h:145-166): FP16 forward, output trimmed and
//                        cast to FP32, element-major [n][n_out]
//   tch_training_step    Trainer::training_step (trainer.h:161-186) with or without the optimizer
//   tch_get_gradients    the trainer's FP16 parameter gradients (trainer.h:230-232), divided by the
//                        static loss scale 128 (trainer.h:171) and widened to FP32
//   tch_loss             Trainer::loss (trainer.h:197-199) of the last step
//
// Every entry point returns 0 on success and -1 on a thrown error, whose message
// tch_last_error() returns.
#include <tiny-cuda-nn/common.h>
#include <tiny-cuda-nn/config.h>
#include <tiny-cuda-nn/encodings/composite.h>
#include <tiny-cuda-nn/encodings/grid.h>

#include <cuda_fp16.h>

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

using tcnn::json;
using precision_t = tcnn::network_precision_t;

// CompositeEncoding keeps its nested encodings private and the reference application never sets a
// per-element max level.  An explicit instantiation may name a private member, so this standard
// idiom hands out a pointer to it without touching the reference headers.
template <typename Tag, typename Tag::type M>
struct Expose {
	friend typename Tag::type member(Tag) { return M; }
};
struct CompositeNested {
	using type = std::vector<std::unique_ptr<tcnn::Encoding<precision_t>>> tcnn::CompositeEncoding<precision_t>::*;
	friend type member(CompositeNested);
};
template struct Expose<CompositeNested, &tcnn::CompositeEncoding<precision_t>::m_nested>;

thread_local std::string g_error;

struct Model {
	tcnn::TrainableModel tm;
	uint32_t n_in = 0, n_out = 0;
	std::unique_ptr<tcnn::Trainer<float, precision_t, precision_t>::ForwardContext> last;
};

tcnn::GridEncoding<precision_t>* find_grid(tcnn::Encoding<precision_t>* e) {
	if (auto* g = dynamic_cast<tcnn::GridEncoding<precision_t>*>(e)) return g;
	if (auto* c = dynamic_cast<tcnn::CompositeEncoding<precision_t>*>(e)) {
		for (auto& n : c->*member(CompositeNested{})) {
			if (auto* g = find_grid(n.get())) return g;
		}
	}
	return nullptr;
}

template <typename F>
int guarded(F&& f) {
	try {
		f();
		return 0;
	} catch (const std::exception& e) {
		g_error = e.what();
		return -1;
	}
}

}  // namespace

extern "C" {

const char* tch_last_error(void) { return g_error.c_str(); }

int tch_create(const char* config_json, uint32_t n_in, uint32_t n_out, void** out) {
	return guarded([&] {
		auto m = std::make_unique<Model>();
		m->tm = tcnn::create_from_config(n_in, n_out, json::parse(config_json));
		m->n_in = n_in;
		m->n_out = n_out;
		*out = m.release();
	});
}

void tch_destroy(void* h) {
	delete static_cast<Model*>(h);
}

size_t tch_n_params(void* h) { return static_cast<Model*>(h)->tm.network->n_params(); }

uint32_t tch_padded_output_width(void* h) { return static_cast<Model*>(h)->tm.network->padded_output_width(); }

uint32_t tch_encoded_width(void* h) {
	return static_cast<Model*>(h)->tm.network->encoding()->padded_output_width();
}

int tch_set_params(void* h, const float* host_params, size_t n) {
	return guarded([&] { static_cast<Model*>(h)->tm.trainer->set_params_full_precision(host_params, n, false); });
}

int tch_get_params(void* h, float* host_params, size_t n) {
	return guarded([&] {
		auto* m = static_cast<Model*>(h);
		if (n != m->tm.network->n_params()) throw std::runtime_error{"tch_get_params: wrong size"};
		CUDA_CHECK_THROW(cudaDeviceSynchronize());
		CUDA_CHECK_THROW(cudaMemcpy(host_params, m->tm.trainer->params_full_precision(), n * sizeof(float), cudaMemcpyDeviceToHost));
	});
}

int tch_set_max_level_gpu(void* h, float* device_levels) {
	return guarded([&] {
		auto* g = find_grid(static_cast<Model*>(h)->tm.network->encoding().get());
		if (!g) throw std::runtime_error{"tch_set_max_level_gpu: no grid encoding"};
		g->set_max_level_gpu(device_levels);
	});
}

int tch_inference(void* h, void* stream, uint32_t n, const float* d_in, float* d_out) {
	return guarded([&] {
		auto* m = static_cast<Model*>(h);
		tcnn::GPUMatrix<float> in{const_cast<float*>(d_in), m->n_in, n};
		tcnn::GPUMatrix<float> out{d_out, m->n_out, n};
		m->tm.network->inference((cudaStream_t)stream, in, out);
	});
}

int tch_training_step(void* h, void* stream, uint32_t n, const float* d_in, const float* d_target, int run_optimizer) {
	return guarded([&] {
		auto* m = static_cast<Model*>(h);
		tcnn::GPUMatrix<float> in{const_cast<float*>(d_in), m->n_in, n};
		tcnn::GPUMatrix<float> target{const_cast<float*>(d_target), m->n_out, n};
		m->last = m->tm.trainer->training_step((cudaStream_t)stream, in, target, nullptr, run_optimizer != 0);
	});
}

int tch_loss(void* h, void* stream, float* loss) {
	return guarded([&] {
		auto* m = static_cast<Model*>(h);
		if (!m->last) throw std::runtime_error{"tch_loss: no training step yet"};
		*loss = m->tm.trainer->loss((cudaStream_t)stream, *m->last);
	});
}

int tch_get_gradients(void* h, float* host_grad, size_t n) {
	return guarded([&] {
		auto* m = static_cast<Model*>(h);
		if (n != m->tm.network->n_params()) throw std::runtime_error{"tch_get_gradients: wrong size"};
		std::vector<precision_t> g(n);
		CUDA_CHECK_THROW(cudaDeviceSynchronize());
		CUDA_CHECK_THROW(cudaMemcpy(g.data(), m->tm.trainer->param_gradients(), n * sizeof(precision_t), cudaMemcpyDeviceToHost));
		for (size_t i = 0; i < n; ++i) host_grad[i] = (float)g[i] / 128.0f;
	});
}

}  // extern "C"
