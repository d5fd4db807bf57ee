// usgb_process_frame_noalloc: one whole frame (signal preparation, then
// delay-and-sum with the coherence factor) without allocating any device
// memory.
//
// Who needs it: callers that must not allocate device memory while they run,
// for example a host that has already handed almost all GPU memory to its own
// pool (a cudaMalloc from this library would fail or fragment that pool), or
// an acquisition loop with a fixed latency budget that cannot absorb
// allocation calls. The normal entry points allocate their buffers in
// usgb_create; this one takes its inputs and outputs from the caller and keeps
// everything else it needs - the filter and FFT tables, the element positions
// and the prepared signal tensor - in one fixed device array declared below.
//
// The array is a file-scope __device__ variable of kNoAllocScratchBytes
// (64 MiB); every GPU that loads the library holds it until the process exits.
// All calls share it and it keeps whatever the last call left there, so each
// call rewrites every part it uses (tables, positions, tensor) and clears the
// device status word before launching. Calls whose GPU work overlaps (on
// different streams, or from different threads) race on the array; the caller
// must order them.
//
// Device-side failures (a bounded wait of the delay-and-sum that gave up, so
// the image is incomplete) are reported through a status word: the caller's
// own device word when it passes one (cleared by the call, set by the kernels,
// read by the caller after the stream completes, so the call stays
// asynchronous), else the call waits for its work on the stream and returns
// USGB_ERR_DEVICE_TIMEOUT itself.
//
// In host code `g_noallocScratch` only stands in for the array: its device
// address is obtained with cudaGetSymbolAddress once per device, with that
// device current, on the first call on that device.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/usgb.h"
#include "usgb_common.cuh"
#include "usgb_internal.h"
#include "usgb_params.h"
#include "usgb_tables.h"

namespace {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;  // 64 MiB

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

std::mutex g_addrMutex;
std::vector<void*> g_scratchAddr;  // per device ordinal; nullptr until looked up

struct Fail {
	int code;
	std::string msg;
};

#define NA_FAIL(CODE, EXPR)                \
	do {                                   \
		std::ostringstream os_;            \
		os_ << EXPR;                       \
		throw Fail{(CODE), os_.str()};     \
	} while (0)

#define NA_CUDA(CALL)                                                                   \
	do {                                                                                \
		const cudaError_t e_ = (CALL);                                                  \
		if (e_ != cudaSuccess) NA_FAIL(USGB_ERR_CUDA, #CALL << ": " << cudaGetErrorString(e_)); \
	} while (0)

// Device address of the scratch array on the current device (looked up once
// per device with cudaGetSymbolAddress).
void* scratch_address()
{
	int dev = 0;
	NA_CUDA(cudaGetDevice(&dev));
	std::lock_guard<std::mutex> lock(g_addrMutex);
	if (g_scratchAddr.size() <= static_cast<size_t>(dev)) g_scratchAddr.resize(dev + 1, nullptr);
	if (!g_scratchAddr[dev]) {
		void* ptr = nullptr;
		NA_CUDA(cudaGetSymbolAddress(&ptr, g_noallocScratch));
		g_scratchAddr[dev] = ptr;
	}
	return g_scratchAddr[dev];
}

// Byte layout of one call inside the scratch array.
struct Layout {
	size_t err, taps, dc, tw, hilb, stw, tx, rx, apod, sig, total;
};

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

int run(const usgb_sta_params* p, const float* d_rf, const float* d_grid, uint32_t ncols, uint32_t nrows,
		float* d_value, float* d_factor, uint32_t* d_status, cudaStream_t stream)
{
	// ---- parameter checks: the same function, rules and messages as usgb_create ----
	usgb::host::FrameConsts k{};
	size_t npix = 0;
	try {
		k = usgb::host::check_frame_params(p);
		npix = usgb::host::check_grid_size(ncols, nrows);
	} catch (const usgb::host::ParamError& e) {
		throw Fail{e.code, e.msg};
	}
	if (!d_rf || !d_grid || !d_value || !d_factor) NA_FAIL(USGB_ERR_INVALID_PARAMETER, "null device pointer");
	const bool analytic = k.analytic;
	const unsigned U = k.U;
	const unsigned L = k.L;
	const unsigned numSignals = p->num_tx * p->num_rx;

	// ---- host tables (no device memory involved) ----
	usgb::host::PolyTaps poly;
	if (!usgb::host::make_poly_taps(analytic, U, poly)) NA_FAIL(USGB_ERR_INVALID_STATE, "FIR length is not 2*U*K + 1");
	usgb::PrepParams pp{};
	usgb::host::FFTTables fft;
	if (analytic) {
		if (!usgb::host::make_fft_tables(L, fft)) NA_FAIL(USGB_ERR_INVALID_STATE, "FFT size not supported");
		usgb::host::set_fft_params(pp, fft);
	}
	const std::vector<float> dc = usgb::host::dc_coefficients(poly, U, p->num_samples, k.deadZone);
	std::vector<float> apod(p->num_rx, 1.0f);
	if (analytic && p->rx_apod) apod.assign(p->rx_apod, p->rx_apod + p->num_rx);

	// ---- scratch layout and size check ----
	const size_t elemBytes = k.elemBytes;
	const unsigned sigStride = k.sigStride;
	Layout lay{};
	size_t off = 0;
	lay.err = off; off = align256(off + sizeof(unsigned));
	lay.taps = off; off = align256(off + poly.poly.size() * sizeof(float));
	lay.dc = off; off = align256(off + dc.size() * sizeof(float));
	lay.tw = off; off = align256(off + fft.tw.size() * sizeof(float2));
	lay.hilb = off; off = align256(off + fft.hilb.size() * sizeof(float4));
	lay.stw = off; off = align256(off + fft.stageTw.size() * sizeof(float2));
	lay.tx = off; off = align256(off + 2 * p->num_tx * sizeof(float));
	lay.rx = off; off = align256(off + 2 * p->num_rx * sizeof(float));
	lay.apod = off; off = align256(off + apod.size() * sizeof(float));
	lay.sig = off; off = align256(off + static_cast<size_t>(numSignals) * sigStride * elemBytes + 256);
	lay.total = off;
	if (lay.total > kNoAllocScratchBytes) {
		NA_FAIL(USGB_ERR_INVALID_VALUE, "Frame too large for the no-allocation entry point: it needs " << lay.total
				<< " bytes of scratch, the fixed array holds " << kNoAllocScratchBytes
				<< " (use usgb_create / usgb_process_device, or FP16/BF16 storage).");
	}

	// ---- device work: everything below writes into the fixed array ----
	unsigned char* base = static_cast<unsigned char*>(scratch_address());
	unsigned* status = d_status ? d_status : reinterpret_cast<unsigned*>(base + lay.err);
	NA_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned), stream));
	NA_CUDA(cudaMemcpyAsync(base + lay.taps, poly.poly.data(), poly.poly.size() * sizeof(float), cudaMemcpyHostToDevice, stream));
	NA_CUDA(cudaMemcpyAsync(base + lay.dc, dc.data(), dc.size() * sizeof(float), cudaMemcpyHostToDevice, stream));
	if (analytic) {
		NA_CUDA(cudaMemcpyAsync(base + lay.tw, fft.tw.data(), fft.tw.size() * sizeof(float2), cudaMemcpyHostToDevice, stream));
		NA_CUDA(cudaMemcpyAsync(base + lay.hilb, fft.hilb.data(), fft.hilb.size() * sizeof(float4), cudaMemcpyHostToDevice, stream));
		if (!fft.stageTw.empty()) {
			NA_CUDA(cudaMemcpyAsync(base + lay.stw, fft.stageTw.data(), fft.stageTw.size() * sizeof(float2),
					cudaMemcpyHostToDevice, stream));
		}
	}
	NA_CUDA(cudaMemcpyAsync(base + lay.tx, p->tx_xy, 2 * p->num_tx * sizeof(float), cudaMemcpyHostToDevice, stream));
	NA_CUDA(cudaMemcpyAsync(base + lay.rx, p->rx_xy, 2 * p->num_rx * sizeof(float), cudaMemcpyHostToDevice, stream));
	NA_CUDA(cudaMemcpyAsync(base + lay.apod, apod.data(), apod.size() * sizeof(float), cudaMemcpyHostToDevice, stream));

	pp.rf = d_rf;
	pp.out = base + lay.sig;
	pp.outStride = sigStride;
	pp.numSignals = numSignals;
	pp.ns = p->num_samples;
	pp.U = U;
	pp.L = L;
	pp.tapsPerPhase = poly.tapsPerPhase;
	pp.tapsStride = poly.tapsStride;
	usgb::host::set_param_taps(pp, poly.poly);
	pp.polyTaps = reinterpret_cast<const float*>(base + lay.taps);
	pp.deadZone = k.deadZone;
	const float scale = k.scale;
	pp.outScale = scale;
	pp.tw = reinterpret_cast<const float2*>(base + lay.tw);
	pp.hilb = reinterpret_cast<const float4*>(base + lay.hilb);
	pp.stw = (analytic && !fft.stageTw.empty()) ? reinterpret_cast<const float2*>(base + lay.stw) : nullptr;

	int dev = 0, maxSmem = 0;
	NA_CUDA(cudaGetDevice(&dev));
	NA_CUDA(cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
	if (pp.stw && usgb::prep_smem_bytes(pp, analytic) > static_cast<size_t>(maxSmem)) pp.stw = nullptr;
	if (usgb::prep_smem_bytes(pp, analytic) > static_cast<size_t>(maxSmem)) {
		NA_FAIL(USGB_ERR_UNSUPPORTED, "A-scan too long for on-chip preparation (signal length " << L << ").");
	}
	// The preparation usgb_create's context chooses: the persistent kernel
	// with the DC removed in the FIR pass where it fits, so both entry points
	// form the same signals.
	pp.dcCoef = reinterpret_cast<const float*>(base + lay.dc);
	pp.errWord = status;
	if (!usgb::prep_uses_stream(pp) || usgb::prep_stream_smem_bytes(pp, analytic) > static_cast<size_t>(maxSmem)) {
		pp.dcCoef = nullptr;
	} else {
		cudaPointerAttributes at{};
		if (pp.ns % 4 == 0 && reinterpret_cast<uintptr_t>(d_rf) % 16 == 0 &&
				cudaPointerGetAttributes(&at, d_rf) == cudaSuccess && at.type == cudaMemoryTypeDevice) {
			pp.rfBulk = 1;
		}
		cudaGetLastError();
	}
	NA_CUDA(usgb::launch_prep(pp, static_cast<int>(p->storage), analytic, stream));

	usgb::DasParams dp{};
	dp.sig = base + lay.sig;
	dp.sigStride = sigStride;
	dp.L = L;
	dp.numTx = p->num_tx;
	dp.numRx = p->num_rx;
	dp.txXY = reinterpret_cast<const float*>(base + lay.tx);
	dp.rxXY = reinterpret_cast<const float*>(base + lay.rx);
	dp.apod = reinterpret_cast<const float*>(base + lay.apod);
	dp.grid = d_grid;
	dp.npix = static_cast<unsigned>(npix);  // <= 2^31 (check_grid_size)
	dp.ncols = ncols;
	dp.nrows = nrows;
	dp.invCT = k.invCT;
	dp.signalOffset = k.signalOffset;
	dp.valueCoef = k.valueCoef;
	dp.invScale = 1.0f / scale;
	dp.pcfFactor = k.pcfFactor;
	dp.scfP = p->scf_p;
	dp.delayMode = USGB_DELAY_AUTO;
	dp.invCTd = static_cast<double>(p->sampling_frequency) * U / p->propagation_speed;
	dp.signalOffsetd = static_cast<double>(p->sampling_frequency) * U * p->peak_offset / p->center_frequency;
	dp.value = d_value;
	dp.factor = d_factor;
	dp.errWord = status;
	dp.tileCols = 32;
	dp.tileRows = 8;
	dp.stageBytes = 16384;
	dp.stages = 4;
	// The staged kernel when its shared memory fits, the plain one otherwise.
	const bool staged = usgb::das_staged_smem_bytes(p->num_tx, p->num_rx, dp.tileRows, dp.stageBytes, dp.stages)
			<= static_cast<size_t>(maxSmem);
	if (!staged && static_cast<size_t>(p->num_tx) * 128 * sizeof(float) > static_cast<size_t>(maxSmem)) {
		NA_FAIL(USGB_ERR_UNSUPPORTED, "Too many transmit elements for the delay table: " << p->num_tx << '.');
	}
	NA_CUDA(usgb::launch_das(dp, static_cast<int>(p->storage), static_cast<int>(p->coherence), analytic,
			staged ? 1 : 0, stream));
	if (!d_status) {
		// No caller word: wait for this frame and read the array's word (a
		// device-to-host copy into a local, then the stream's completion).
		unsigned word = 0;
		NA_CUDA(cudaMemcpyAsync(&word, status, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
		NA_CUDA(cudaStreamSynchronize(stream));
		if (word & usgb::DEVERR_WAIT_TIMEOUT) {
			NA_FAIL(USGB_ERR_DEVICE_TIMEOUT, "A delay-and-sum wait gave up on the device; the image is incomplete.");
		}
		if (word) NA_FAIL(USGB_ERR_INVALID_STATE, "Device-side error " << word << " in the delay-and-sum.");
	}
	return USGB_OK;
}

}  // namespace

extern "C" int usgb_process_frame_noalloc(const usgb_sta_params* params, const float* d_rf, const float* d_grid_xyz,
		uint32_t ncols, uint32_t nrows, float* d_value, float* d_factor, uint32_t* d_status, void* cuda_stream,
		char* error_message, size_t error_capacity)
{
	std::string msg;
	int rc = USGB_OK;
	try {
		rc = run(params, d_rf, d_grid_xyz, ncols, nrows, d_value, d_factor, d_status,
				static_cast<cudaStream_t>(cuda_stream));
	} catch (const Fail& f) {
		msg = f.msg;
		rc = f.code;
	} catch (const std::exception& e) {
		msg = e.what();
		rc = USGB_ERR_INVALID_STATE;
	}
	if (error_message && error_capacity > 0) {
		const size_t n = std::min(msg.size(), error_capacity - 1);
		std::memcpy(error_message, msg.data(), n);
		error_message[n] = '\0';
	}
	return rc;
}
