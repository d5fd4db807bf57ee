// Image post-processing after the delay-and-sum: the envelope along each
// image column and the conversion to decibels, as the reference computes them
// for its "Envelope - dB" / "Rectified - dB" images:
//   ParallelHilbertEnvelope<float>::calculateDim2Value  src/parallel/ParallelHilbertEnvelope.h:83-95
//     (HilbertEnvelope::calculate per column, src/util/HilbertEnvelope.h:211-232)
//   Util::linearToDecibels(std::vector<T>&, T)          src/util/Util.h:600-613
// The envelope reuses the preparation kernel's Hilbert transform (same FFT
// size rule, N = max(nextFastEvenSize(n + 1024), 2048)) on the image columns;
// the decibel conversion is a max-magnitude reduction and one elementwise
// pass.
#include <algorithm>
#include <cmath>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/usgb.h"
#include "usgb_common.cuh"
#include "usgb_internal.h"
#include "usgb_tables.h"

namespace {

constexpr int kPostThreads = 256;

// Largest |v| as the bits of a non-negative float (ordered like the floats).
__global__ void __launch_bounds__(kPostThreads)
max_abs_kernel(const float* __restrict__ data, size_t n, unsigned* __restrict__ maxBits)
{
	float m = 0.f;
	for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
			i += static_cast<size_t>(gridDim.x) * blockDim.x) {
		m = fmaxf(m, fabsf(data[i]));
	}
	for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(maxBits, __float_as_uint(m));
}

// v *= 1 / max|v| (unless the maximum is 0), then 20 log10(v), or minDb at or
// below minVal = 10^(minDb / 20).
__global__ void __launch_bounds__(kPostThreads)
decibels_kernel(float* __restrict__ data, size_t n, const unsigned* __restrict__ maxBits, float minDb, float minVal)
{
	const float maxAbs = __uint_as_float(*maxBits);
	const float coeff = (maxAbs != 0.f) ? 1.0f / maxAbs : 1.0f;
	for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
			i += static_cast<size_t>(gridDim.x) * blockDim.x) {
		const float v = (maxAbs != 0.f) ? data[i] * coeff : data[i];
		data[i] = (v <= minVal) ? minDb : 20.0f * log10f(v);
	}
}

struct PostFailure {
	int code;
	std::string msg;
};

#define POST_FAIL(CODE, STREAM_EXPR)          \
	do {                                      \
		std::ostringstream os_;               \
		os_ << STREAM_EXPR;                   \
		throw PostFailure{(CODE), os_.str()}; \
	} while (0)

#define POST_CUDA(CALL)                                                                                  \
	do {                                                                                                 \
		const cudaError_t e_ = (CALL);                                                                   \
		if (e_ != cudaSuccess) {                                                                         \
			POST_FAIL(e_ == cudaErrorMemoryAllocation ? USGB_ERR_OUT_OF_MEMORY : USGB_ERR_CUDA,            \
					#CALL << ": " << cudaGetErrorString(e_));                                            \
		}                                                                                                \
	} while (0)

thread_local std::string g_postCreateError;

}  // namespace

struct usgb_post {
	unsigned numSamples = 0;
	usgb::host::FFTTables fft;
	float* d_taps = nullptr;
	float2* d_tw = nullptr;
	float4* d_hilb = nullptr;
	float2* d_stw = nullptr;
	unsigned* d_max = nullptr;
	bool stageTw = true;
	unsigned numSMs = 0;
	std::string err;

	~usgb_post()
	{
		void* dev[] = {d_taps, d_tw, d_hilb, d_stw, d_max};
		for (void* p : dev) if (p) cudaFree(p);
	}
};

namespace {

template<typename F>
int post_guarded(usgb_post* p, F&& f)
{
	if (!p) return USGB_ERR_INVALID_PARAMETER;
	try {
		f();
		return USGB_OK;
	} catch (const PostFailure& e) {
		p->err = e.msg;
		return e.code;
	}
}

usgb::PrepParams envelope_params(const usgb_post* p, const float* in, float* out, unsigned columns)
{
	usgb::PrepParams pp{};
	pp.rf = in;
	pp.out = out;
	pp.outStride = p->numSamples;
	pp.numSignals = columns;
	pp.ns = p->numSamples;
	pp.U = 1;
	pp.L = p->numSamples;
	pp.tapsPerPhase = 1;
	pp.tapsStride = 4;
	pp.polyTaps = p->d_taps;
	pp.deadZone = 0;
	pp.outScale = 1.0f;
	usgb::host::set_fft_params(pp, p->fft);
	pp.tw = p->d_tw;
	pp.hilb = p->d_hilb;
	pp.stw = p->stageTw ? p->d_stw : nullptr;
	return pp;
}

}  // namespace

extern "C" {

int usgb_post_create(uint32_t num_samples, usgb_post** out)
{
	if (!out) return USGB_ERR_INVALID_PARAMETER;
	*out = nullptr;
	usgb_post* p = nullptr;
	try {
		if (num_samples == 0) POST_FAIL(USGB_ERR_INVALID_PARAMETER, "The number of input samples (0) is = 0.");
		if (num_samples > (1u << 20)) {
			POST_FAIL(USGB_ERR_INVALID_PARAMETER, "The number of input samples (" << num_samples << ") is greater than "
					<< (1u << 20) << '.');
		}
		p = new usgb_post();
		p->numSamples = num_samples;
		if (!usgb::host::make_fft_tables(num_samples, p->fft)) POST_FAIL(USGB_ERR_INVALID_STATE, "FFT size not supported");
		const float taps[4] = {1.0f, 0.f, 0.f, 0.f};
		POST_CUDA(cudaMalloc(&p->d_taps, sizeof(taps)));
		POST_CUDA(cudaMemcpy(p->d_taps, taps, sizeof(taps), cudaMemcpyHostToDevice));
		auto upload = [](auto** dst, const auto& v) {
			using E = typename std::decay_t<decltype(v)>::value_type;
			POST_CUDA(cudaMalloc(dst, std::max<size_t>(v.size(), 1) * sizeof(E)));
			if (!v.empty()) POST_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(E), cudaMemcpyHostToDevice));
		};
		upload(&p->d_tw, p->fft.tw);
		upload(&p->d_hilb, p->fft.hilb);
		upload(&p->d_stw, p->fft.stageTw);
		POST_CUDA(cudaMalloc(&p->d_max, sizeof(unsigned)));
		int dev = 0, maxSmem = 0, sms = 0;
		POST_CUDA(cudaGetDevice(&dev));
		POST_CUDA(cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
		POST_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
		p->numSMs = static_cast<unsigned>(sms);
		if (usgb::prep_smem_bytes(envelope_params(p, nullptr, nullptr, 0), true) > static_cast<size_t>(maxSmem)) {
			p->stageTw = false;
			if (usgb::prep_smem_bytes(envelope_params(p, nullptr, nullptr, 0), true) > static_cast<size_t>(maxSmem)) {
				POST_FAIL(USGB_ERR_UNSUPPORTED, "Columns of " << num_samples << " samples are too long for the on-chip envelope.");
			}
		}
		*out = p;
		return USGB_OK;
	} catch (const PostFailure& e) {
		g_postCreateError = e.msg;
		delete p;
		return e.code;
	}
}

void usgb_post_destroy(usgb_post* p)
{
	delete p;
}

const char* usgb_post_last_error(const usgb_post* p)
{
	return p ? p->err.c_str() : g_postCreateError.c_str();
}

int usgb_post_envelope_device(usgb_post* p, const float* d_in, float* d_out, uint32_t num_columns, void* stream)
{
	return post_guarded(p, [&] {
		if (!d_in || !d_out) POST_FAIL(USGB_ERR_INVALID_PARAMETER, "null device pointer");
		if (num_columns == 0) return;
		POST_CUDA(usgb::launch_envelope(envelope_params(p, d_in, d_out, num_columns), static_cast<cudaStream_t>(stream)));
	});
}

int usgb_post_decibels_device(usgb_post* p, float* d_data, size_t n, float min_db, void* stream)
{
	return post_guarded(p, [&] {
		if (!d_data) POST_FAIL(USGB_ERR_INVALID_PARAMETER, "null device pointer");
		if (n == 0) return;
		const cudaStream_t st = static_cast<cudaStream_t>(stream);
		// decibelsToLinear(minDecibels) in float, as Util::linearToDecibels<float>.
		const float minVal = std::pow(10.0f, min_db * 0.05f);
		const size_t want = (n + kPostThreads - 1) / kPostThreads;
		const unsigned blocks = static_cast<unsigned>(std::min<size_t>(want, static_cast<size_t>(p->numSMs) * 8));
		POST_CUDA(cudaMemsetAsync(p->d_max, 0, sizeof(unsigned), st));
		max_abs_kernel<<<blocks, kPostThreads, 0, st>>>(d_data, n, p->d_max);
		POST_CUDA(cudaGetLastError());
		decibels_kernel<<<blocks, kPostThreads, 0, st>>>(d_data, n, p->d_max, min_db, minVal);
		POST_CUDA(cudaGetLastError());
	});
}

}  // extern "C"
