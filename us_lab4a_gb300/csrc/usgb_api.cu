// C-ABI implementation of libusgb: parameter checks (with the reference's
// error semantics), FIR/FFT table construction, device buffers and the
// per-frame launch sequence (signal preparation, then delay-and-sum).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/usgb.h"
#include "usgb_common.cuh"
#include "usgb_internal.h"
#include "usgb_params.h"
#include "usgb_tables.h"

namespace {

using usgb::host::kPi;

thread_local std::string g_createError;

struct Failure {
	int code;
	std::string msg;
};

#define USGB_FAIL(CODE, STREAM_EXPR)            \
	do {                                        \
		std::ostringstream os_;                 \
		os_ << STREAM_EXPR;                     \
		throw Failure{(CODE), os_.str()};       \
	} while (0)

#define USGB_CUDA(CALL)                                                                       \
	do {                                                                                      \
		const cudaError_t e_ = (CALL);                                                        \
		if (e_ != cudaSuccess) {                                                              \
			USGB_FAIL(e_ == cudaErrorMemoryAllocation ? USGB_ERR_OUT_OF_MEMORY : USGB_ERR_CUDA, \
					#CALL << ": " << cudaGetErrorString(e_));                                 \
		}                                                                                     \
	} while (0)

}  // namespace

struct usgb_ctx {
	usgb_sta_params prm{};
	std::vector<float> txXY, rxXY, apod;
	unsigned numSignals = 0, L = 0, U = 1, deadZone = 0, tapsPerPhase = 1, tapsStride = 4;
	usgb::host::FFTTables fft;   // Hilbert FFT plan (analytic path)
	bool stageTw = false;        // per-stage twiddle tables fit in shared memory
	unsigned sigStride = 0;
	size_t sigBytes = 0;
	size_t elemBytes = 0;
	float invCT = 0, signalOffset = 0, valueCoef = 0, pcfFactor = 0, scale = 1;
	bool analytic = true;

	float* d_txXY = nullptr;
	float* d_rxXY = nullptr;
	float* d_apod = nullptr;
	float* d_polyTaps = nullptr;
	std::vector<float> polyHost;   // the same taps, for the launch parameters
	float* d_dcCoef = nullptr;     // DC weights of the input samples (usgb::host::dc_coefficients)
	bool prepStream = false;       // the persistent preparation kernel fits in shared memory
	float2* d_tw = nullptr;
	float4* d_hilb = nullptr;
	float2* d_stw = nullptr;
	float* d_rf = nullptr;
	void* d_sig = nullptr;
	float* d_grid = nullptr;
	float* d_value = nullptr;
	float* d_factor = nullptr;
	unsigned* d_err = nullptr;
	size_t gridCap = 0;
	unsigned ncols = 0, nrows = 0, npix = 0;
	bool gridSet = false;

	float* h_rf = nullptr;  // pinned staging of submitted RF
	float* h_out = nullptr; // pinned staging of value/factor
	size_t hOutCap = 0;
	std::vector<unsigned char> submitted;

	cudaStream_t stream = nullptr;
	bool ownStream = false;
	bool hostDirectAvailable = false;  // kernels can read/write pageable host memory (host page tables)
	bool hostDirect = false;
	int dasVariant = 0;
	bool dasExplicit = false;   // chosen by usgb_set_das_variant / usgb_autotune_das: kept when the grid changes
	int delayMode = USGB_DELAY_AUTO;
	unsigned tileRows = 8;
	unsigned stageBytes = 16384;
	unsigned stages = 4;
	unsigned long long waitLimitNs = 0;   // usgb_set_wait_test: 0 = the kernels' 2 s
	unsigned testSkipStage = 0;           // usgb_set_wait_test: 0 = none
	std::string err;

	~usgb_ctx()
	{
		void* dev[] = {d_txXY, d_rxXY, d_apod, d_polyTaps, d_dcCoef, d_tw, d_hilb, d_stw, d_rf, d_sig, d_grid, d_value, d_factor, d_err};
		for (void* p : dev) if (p) cudaFree(p);
		if (h_rf) cudaFreeHost(h_rf);
		if (h_out) cudaFreeHost(h_out);
		if (ownStream && stream) cudaStreamDestroy(stream);
	}
};

struct usgb_batch {
	unsigned maxFrames = 0, maxElements = 0, maxSignalLength = 0;
	int dasVariant = 2;      // 1: staged kernel, 2: receiver-group kernel
	unsigned tileRows = 4, stageBytes = 32768, stages = 2;
	unsigned numSMs = 0;
	size_t descBytes = 0;
	unsigned char* h_desc = nullptr;   // pinned: header, prep frames, DAS frames
	unsigned char* d_desc = nullptr;
	unsigned* d_err = nullptr;
	cudaEvent_t done = nullptr;
	bool pending = false;
	// Captured graph and the launch shape it was captured for.
	cudaGraphExec_t graph = nullptr;
	size_t graphPrepSmem = 0;
	unsigned graphPrepBlocks = 0, graphDasBlocks = 0;
	int graphStorage = -1;
	bool graphAnalytic = true;
	cudaStream_t graphStream = nullptr;
	std::string err;

	~usgb_batch()
	{
		if (graph) cudaGraphExecDestroy(graph);
		if (done) cudaEventDestroy(done);
		if (d_desc) cudaFree(d_desc);
		if (d_err) cudaFree(d_err);
		if (h_desc) cudaFreeHost(h_desc);
	}
};

namespace {

void build_tables(usgb_ctx* c)
{
	usgb::host::PolyTaps poly;
	if (!usgb::host::make_poly_taps(c->analytic, c->U, poly)) {
		USGB_FAIL(USGB_ERR_INVALID_STATE, "FIR length is not 2*U*K + 1 for upsampling " << c->U);
	}
	c->tapsPerPhase = poly.tapsPerPhase;
	c->tapsStride = poly.tapsStride;
	c->polyHost = poly.poly;
	USGB_CUDA(cudaMalloc(&c->d_polyTaps, poly.poly.size() * sizeof(float)));
	USGB_CUDA(cudaMemcpy(c->d_polyTaps, poly.poly.data(), poly.poly.size() * sizeof(float), cudaMemcpyHostToDevice));
	const std::vector<float> dc = usgb::host::dc_coefficients(poly, c->U, c->prm.num_samples, c->deadZone);
	USGB_CUDA(cudaMalloc(&c->d_dcCoef, dc.size() * sizeof(float)));
	USGB_CUDA(cudaMemcpy(c->d_dcCoef, dc.data(), dc.size() * sizeof(float), cudaMemcpyHostToDevice));

	if (!c->analytic) return;
	usgb::host::FFTTables& t = c->fft;
	if (!usgb::host::make_fft_tables(c->L, t)) USGB_FAIL(USGB_ERR_INVALID_STATE, "FFT size " << t.M << " not supported");
	auto upload = [](auto** dst, const auto& v) {
		using E = typename std::decay_t<decltype(v)>::value_type;
		USGB_CUDA(cudaMalloc(dst, std::max<size_t>(v.size(), 1) * sizeof(E)));
		if (!v.empty()) USGB_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(E), cudaMemcpyHostToDevice));
	};
	upload(&c->d_tw, t.tw);
	upload(&c->d_hilb, t.hilb);
	upload(&c->d_stw, t.stageTw);
	c->stageTw = true;  // cleared by check_prep_fits when the tables do not fit
}

// ParamError (the shared checks of usgb_params.h) as this file's Failure.
template<typename F>
auto rethrow_param_error(F&& f) -> decltype(f())
{
	try {
		return f();
	} catch (const usgb::host::ParamError& e) {
		throw Failure{e.code, e.msg};
	}
}

void check_and_derive(usgb_ctx* c, const usgb_sta_params* p)
{
	const usgb::host::FrameConsts k = rethrow_param_error([&] { return usgb::host::check_frame_params(p); });
	c->analytic = k.analytic;
	c->prm = *p;
	c->prm.tx_xy = c->prm.rx_xy = c->prm.rx_apod = nullptr;
	c->U = k.U;
	c->numSignals = k.numSignals;
	c->L = k.L;
	c->deadZone = k.deadZone;
	c->invCT = k.invCT;
	c->signalOffset = k.signalOffset;
	c->valueCoef = k.valueCoef;
	c->pcfFactor = k.pcfFactor;
	c->scale = k.scale;

	c->txXY.assign(p->tx_xy, p->tx_xy + 2 * p->num_tx);
	c->rxXY.assign(p->rx_xy, p->rx_xy + 2 * p->num_rx);
	if (p->rx_apod && c->analytic) {
		c->apod.assign(p->rx_apod, p->rx_apod + p->num_rx);
	} else {
		c->apod.assign(p->num_rx, 1.0f);  // the real-RF path has no apodization
	}
	c->elemBytes = k.elemBytes;
	c->sigStride = k.sigStride;
	c->sigBytes = static_cast<size_t>(c->numSignals) * c->sigStride * c->elemBytes + 256;
}

void alloc_frame(usgb_ctx* c)
{
	const usgb_sta_params& p = c->prm;
	USGB_CUDA(cudaMalloc(&c->d_txXY, c->txXY.size() * sizeof(float)));
	USGB_CUDA(cudaMalloc(&c->d_rxXY, c->rxXY.size() * sizeof(float)));
	USGB_CUDA(cudaMalloc(&c->d_apod, c->apod.size() * sizeof(float)));
	USGB_CUDA(cudaMemcpy(c->d_txXY, c->txXY.data(), c->txXY.size() * sizeof(float), cudaMemcpyHostToDevice));
	USGB_CUDA(cudaMemcpy(c->d_rxXY, c->rxXY.data(), c->rxXY.size() * sizeof(float), cudaMemcpyHostToDevice));
	USGB_CUDA(cudaMemcpy(c->d_apod, c->apod.data(), c->apod.size() * sizeof(float), cudaMemcpyHostToDevice));
	const size_t rfBytes = static_cast<size_t>(c->numSignals) * p.num_samples * sizeof(float);
	USGB_CUDA(cudaMalloc(&c->d_rf, rfBytes));
	USGB_CUDA(cudaMalloc(&c->d_sig, c->sigBytes));
	USGB_CUDA(cudaMemset(c->d_sig, 0, c->sigBytes));
	USGB_CUDA(cudaMalloc(&c->d_err, sizeof(unsigned)));
	USGB_CUDA(cudaMemset(c->d_err, 0, sizeof(unsigned)));
	USGB_CUDA(cudaMallocHost(&c->h_rf, rfBytes));
	c->submitted.assign(p.num_tx, 0);
}

usgb::PrepParams prep_params(const usgb_ctx* c, const float* d_rf, void* d_sig)
{
	usgb::PrepParams pp{};
	pp.rf = d_rf;
	pp.out = d_sig;
	pp.outStride = c->sigStride;
	pp.numSignals = c->numSignals;
	pp.ns = c->prm.num_samples;
	pp.U = c->U;
	pp.L = c->L;
	pp.tapsPerPhase = c->tapsPerPhase;
	pp.tapsStride = c->tapsStride;
	pp.polyTaps = c->d_polyTaps;
	usgb::host::set_param_taps(pp, c->polyHost);
	pp.deadZone = c->deadZone;
	pp.outScale = c->scale;
	pp.errWord = c->d_err;
	if (c->prepStream) {
		pp.dcCoef = c->d_dcCoef;
		// Bulk copies of the RF rows need device memory and 16-byte rows (a
		// host pointer read through the host's page tables takes plain loads).
		cudaPointerAttributes at{};
		if (d_rf && pp.ns % 4 == 0 && reinterpret_cast<uintptr_t>(d_rf) % 16 == 0 &&
				cudaPointerGetAttributes(&at, d_rf) == cudaSuccess && at.type == cudaMemoryTypeDevice) {
			pp.rfBulk = 1;
		}
		cudaGetLastError();   // a failed attribute query leaves no error behind
	}
	if (c->analytic) {
		usgb::host::set_fft_params(pp, c->fft);
		pp.tw = c->d_tw;
		pp.hilb = c->d_hilb;
		pp.stw = c->stageTw ? c->d_stw : nullptr;
	}
	return pp;
}

usgb::DasParams das_params(const usgb_ctx* c, const void* d_sig, float* d_value, float* d_factor)
{
	usgb::DasParams dp{};
	dp.sig = d_sig;
	dp.sigStride = c->sigStride;
	dp.L = c->L;
	dp.numTx = c->prm.num_tx;
	dp.numRx = c->prm.num_rx;
	dp.txXY = c->d_txXY;
	dp.rxXY = c->d_rxXY;
	dp.apod = c->d_apod;
	dp.grid = c->d_grid;
	dp.npix = c->npix;
	dp.ncols = c->ncols;
	dp.nrows = c->nrows;
	dp.invCT = c->invCT;
	dp.signalOffset = c->signalOffset;
	dp.valueCoef = c->valueCoef;
	dp.invScale = 1.0f / c->scale;
	dp.pcfFactor = c->pcfFactor;
	dp.scfP = c->prm.scf_p;
	dp.delayMode = c->delayMode;
	{
		const double upFs = static_cast<double>(c->prm.sampling_frequency) * c->U;
		dp.invCTd = upFs / c->prm.propagation_speed;
		dp.signalOffsetd = upFs * c->prm.peak_offset / c->prm.center_frequency;
	}
	dp.value = d_value;
	dp.factor = d_factor;
	dp.errWord = c->d_err;
	dp.tileCols = usgb::das_tile_cols(c->dasVariant);
	dp.pointsPerThread = usgb::das_points_per_thread(c->dasVariant);
	dp.tileRows = c->tileRows;
	dp.stageBytes = c->stageBytes;
	dp.stages = c->stages;
	dp.waitLimitNs = c->waitLimitNs;
	dp.testSkipStage = c->testSkipStage;
	return dp;
}

void choose_grid_das(usgb_ctx* c);

void ensure_grid(usgb_ctx* c, uint32_t ncols, uint32_t nrows)
{
	const size_t npix = rethrow_param_error([&] { return usgb::host::check_grid_size(ncols, nrows); });
	if (npix > c->gridCap) {
		if (c->d_grid) { cudaFree(c->d_grid); c->d_grid = nullptr; }
		if (c->d_value) { cudaFree(c->d_value); c->d_value = nullptr; }
		if (c->d_factor) { cudaFree(c->d_factor); c->d_factor = nullptr; }
		c->gridCap = 0;
		USGB_CUDA(cudaMalloc(&c->d_grid, npix * 3 * sizeof(float)));
		USGB_CUDA(cudaMalloc(&c->d_value, npix * sizeof(float)));
		USGB_CUDA(cudaMalloc(&c->d_factor, npix * sizeof(float)));
		c->gridCap = npix;
	}
	c->ncols = ncols;
	c->nrows = nrows;
	c->npix = static_cast<unsigned>(npix);
	if (!c->dasExplicit) choose_grid_das(c);
}

size_t max_smem()
{
	int dev = 0, v = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return 0;
	if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
	return static_cast<size_t>(v);
}

// Shared memory of a delay-and-sum configuration (variants 1-3).
size_t das_smem_bytes(const usgb_ctx* c, int variant, unsigned rows, unsigned cap, unsigned nst)
{
	return variant >= 2 ? usgb::das_group_smem_bytes(c->prm.num_tx, c->prm.num_rx, usgb::das_tile_cols(variant), rows, cap, nst)
	                    : usgb::das_staged_smem_bytes(c->prm.num_tx, c->prm.num_rx, rows, cap, nst);
}

// Default delay-and-sum kernel before a grid is known: the receiver-group
// kernel on 32 x 4 tiles with 2 stages of 32, 16 or 8 KiB, whichever fits;
// else the staged kernel with 32 x 8 (then 32 x 4) tiles, 16 KiB stages and
// the deepest pipeline that fits; else the plain kernel.
void choose_default_das(usgb_ctx* c)
{
	for (unsigned cap : {32768u, 16384u, 8192u}) {
		if (das_smem_bytes(c, 2, 4u, cap, 2u) <= max_smem()) {
			c->dasVariant = 2;
			c->tileRows = 4;
			c->stageBytes = cap;
			c->stages = 2;
			return;
		}
	}
	for (unsigned rows : {8u, 4u}) {
		for (unsigned nst : {8u, 6u, 4u, 2u}) {
			if (usgb::das_staged_smem_bytes(c->prm.num_tx, c->prm.num_rx, rows, 16384u, nst) <= max_smem()) {
				c->dasVariant = 1;
				c->tileRows = rows;
				c->stageBytes = 16384u;
				c->stages = nst;
				return;
			}
		}
	}
	c->dasVariant = 0;
}

// With the grid known: 64 x 16 tiles of two points per thread (variant 4,
// 2 x 100 KiB stages; cf2d FP32 1.645 ms, FP16 1.12 ms) where the grid gives
// at least 1.5 such tiles per SM; else 64-column tiles of one point per
// thread where the grid gives at least two tiles per SM — 64 x 8 with 2 x 100
// or 96 KiB stages (one block per SM; cf2d 1.77 / 1.80 ms), else 64 x 4 with
// 2 x 48 KiB (1.85 ms; 32 x 4 with 2 x 32 KiB: 1.97 ms) — wherever the
// shared memory fits; else the creation-time default.
void choose_grid_das(usgb_ctx* c)
{
	choose_default_das(c);
	if (c->dasVariant != 2) return;
	int dev = 0, sms = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return;
	if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return;
	const size_t colTiles = (c->ncols + 63) / 64;
	const size_t tiles16 = colTiles * ((c->nrows + 15) / 16);
	if (2 * tiles16 >= 3u * static_cast<size_t>(sms) && das_smem_bytes(c, 4, 8u, 102400u, 2u) <= max_smem()) {
		// 64 x 2R tiles, R in [5, 8] thread rows: the fewest waves of tiles
		// (one block per SM) times the rows of a tile, plus about 0.6 row of
		// set-up per tile (cf2d, 512 rows: R = 7, 296 tiles in 2 waves against
		// 256 tiles of R = 8 in 1.7 waves, which take 2 full waves).
		unsigned bestR = 8;
		double bestCost = 1e30;
		for (unsigned R = 8; R >= 5; --R) {
			const size_t tiles = colTiles * ((c->nrows + 2 * R - 1) / (2 * R));
			const double waves = std::ceil(static_cast<double>(tiles) / sms);
			const double cost = waves * (R + 0.6);
			if (cost < bestCost - 1e-9) {
				bestCost = cost;
				bestR = R;
			}
		}
		c->dasVariant = 4;
		c->tileRows = bestR;
		c->stageBytes = 102400u;
		c->stages = 2;
		return;
	}
	struct Shape { unsigned rows, cap; };
	for (const Shape sh : {Shape{8u, 102400u}, Shape{8u, 98304u}, Shape{4u, 49152u}, Shape{4u, 32768u}}) {
		const size_t tiles = colTiles * ((c->nrows + sh.rows - 1) / sh.rows);
		if (tiles >= 2u * static_cast<size_t>(sms) && das_smem_bytes(c, 3, sh.rows, sh.cap, 2u) <= max_smem()) {
			c->dasVariant = 3;
			c->tileRows = sh.rows;
			c->stageBytes = sh.cap;
			c->stages = 2;
			return;
		}
	}
}

void check_prep_fits(usgb_ctx* c)
{
	int dev = 0, maxSmem = 0;
	USGB_CUDA(cudaGetDevice(&dev));
	USGB_CUDA(cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
	size_t need = usgb::prep_smem_bytes(prep_params(c, nullptr, nullptr), c->analytic);
	if (c->stageTw && need > static_cast<size_t>(maxSmem)) {
		c->stageTw = false;  // every FFT stage reads the two-level table instead
		need = usgb::prep_smem_bytes(prep_params(c, nullptr, nullptr), c->analytic);
	}
	if (need > static_cast<size_t>(maxSmem)) {
		USGB_FAIL(USGB_ERR_UNSUPPORTED, "A-scan too long for on-chip preparation: needs " << need
				<< " bytes of shared memory, the device offers " << maxSmem << " (signal length " << c->L << ").");
	}
	// The persistent kernel holds a second RF row and the DC weights as well.
	c->prepStream = true;
	const usgb::PrepParams sp = prep_params(c, nullptr, nullptr);
	c->prepStream = usgb::prep_uses_stream(sp) && usgb::prep_stream_smem_bytes(sp, c->analytic) <= static_cast<size_t>(maxSmem);
	const size_t dasSmem = static_cast<size_t>(c->prm.num_tx) * 128 * sizeof(float);
	if (dasSmem > static_cast<size_t>(maxSmem)) {
		USGB_FAIL(USGB_ERR_UNSUPPORTED, "Too many transmit elements for the delay table: " << c->prm.num_tx << '.');
	}
}

void run_frame(usgb_ctx* c, const float* d_rf, float* d_value, float* d_factor)
{
	if (!c->gridSet) USGB_FAIL(USGB_ERR_INVALID_STATE, "The grid has not been set.");
	USGB_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
	const usgb::PrepParams pp = prep_params(c, d_rf, c->d_sig);
	USGB_CUDA(usgb::launch_prep(pp, static_cast<int>(c->prm.storage), c->analytic, c->stream));
	const usgb::DasParams dp = das_params(c, c->d_sig, d_value, d_factor);
	USGB_CUDA(usgb::launch_das(dp, static_cast<int>(c->prm.storage), static_cast<int>(c->prm.coherence),
			c->analytic, c->dasVariant, c->stream));
}

template<typename F>
int guarded(usgb_ctx* c, F&& f)
{
	if (!c) return USGB_ERR_INVALID_PARAMETER;
	try {
		f();
		return USGB_OK;
	} catch (const Failure& e) {
		c->err = e.msg;
		return e.code;
	} catch (const std::bad_alloc&) {
		c->err = "host allocation failed";
		return USGB_ERR_OUT_OF_MEMORY;
	} catch (const std::exception& e) {
		c->err = e.what();
		return USGB_ERR_INVALID_STATE;
	}
}

}  // namespace

extern "C" {

const char* usgb_version(void) { return "usgb 0.1 (sm_103a)"; }

int usgb_create(const usgb_sta_params* params, usgb_ctx** out)
{
	if (!out) {
		g_createError = "null output pointer";
		return USGB_ERR_INVALID_PARAMETER;
	}
	*out = nullptr;
	usgb_ctx* c = nullptr;
	try {
		c = new usgb_ctx();
		check_and_derive(c, params);
		build_tables(c);
		check_prep_fits(c);
		choose_default_das(c);
		alloc_frame(c);
		{
			int dev = 0, pageable = 0, hostTables = 0;
			USGB_CUDA(cudaGetDevice(&dev));
			USGB_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
			USGB_CUDA(cudaDeviceGetAttribute(&hostTables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
			c->hostDirectAvailable = pageable && hostTables;
			c->hostDirect = c->hostDirectAvailable;
		}
		USGB_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
		c->ownStream = true;
		*out = c;
		return USGB_OK;
	} catch (const Failure& e) {
		g_createError = e.msg;
		delete c;
		return e.code;
	} catch (const std::bad_alloc&) {
		g_createError = "host allocation failed";
		delete c;
		return USGB_ERR_OUT_OF_MEMORY;
	}
}

void usgb_destroy(usgb_ctx* c)
{
	if (!c) return;
	if (c->stream) cudaStreamSynchronize(c->stream);
	delete c;
}

const char* usgb_last_error(const usgb_ctx* c)
{
	return c ? c->err.c_str() : g_createError.c_str();
}

int usgb_set_stream(usgb_ctx* c, void* s)
{
	return guarded(c, [&] {
		// Work queued on the previous stream (e.g. RF transfers started by
		// usgb_submit_rf) finishes before the context moves.
		if (c->stream) USGB_CUDA(cudaStreamSynchronize(c->stream));
		if (c->ownStream && c->stream) USGB_CUDA(cudaStreamDestroy(c->stream));
		c->ownStream = false;
		c->stream = static_cast<cudaStream_t>(s);
	});
}

int usgb_set_grid(usgb_ctx* c, const float* xyz, uint32_t ncols, uint32_t nrows)
{
	return guarded(c, [&] {
		if (!xyz) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "null grid");
		ensure_grid(c, ncols, nrows);
		USGB_CUDA(cudaMemcpyAsync(c->d_grid, xyz, static_cast<size_t>(c->npix) * 3 * sizeof(float),
				cudaMemcpyHostToDevice, c->stream));
		USGB_CUDA(cudaStreamSynchronize(c->stream));
		c->gridSet = true;
	});
}

int usgb_set_grid_device(usgb_ctx* c, const float* d_xyz, uint32_t ncols, uint32_t nrows)
{
	return guarded(c, [&] {
		if (!d_xyz) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "null grid");
		ensure_grid(c, ncols, nrows);
		USGB_CUDA(cudaMemcpyAsync(c->d_grid, d_xyz, static_cast<size_t>(c->npix) * 3 * sizeof(float),
				cudaMemcpyDeviceToDevice, c->stream));
		c->gridSet = true;
	});
}

int usgb_submit_rf(usgb_ctx* c, uint32_t tx, const float* rf, uint32_t num_rx, uint32_t num_samples)
{
	return guarded(c, [&] {
		if (!rf) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "null RF");
		if (tx >= c->prm.num_tx) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid tx index: " << tx << '.');
		if (num_rx != c->prm.num_rx || num_samples != c->prm.num_samples) {
			USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Data size mismatch.");
		}
		const size_t n = static_cast<size_t>(num_rx) * num_samples;
		float* staged = c->h_rf + static_cast<size_t>(tx) * n;
		std::memcpy(staged, rf, n * sizeof(float));
		// The transfer of this transmit event starts now, on the context's
		// stream, while the caller copies the next one (usgb_process waits for
		// the stream before it returns, so the staging area is free again by
		// the next frame; a repeated submission is transferred again, after the
		// first, in stream order).
		USGB_CUDA(cudaMemcpyAsync(c->d_rf + static_cast<size_t>(tx) * n, staged, n * sizeof(float),
				cudaMemcpyHostToDevice, c->stream));
		c->submitted[tx] = 1;
	});
}

int usgb_process(usgb_ctx* c, float* value, float* factor)
{
	return guarded(c, [&] {
		if (!value) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "null value output");
		for (unsigned t = 0; t < c->prm.num_tx; ++t) {
			if (!c->submitted[t]) USGB_FAIL(USGB_ERR_INVALID_STATE, "RF of tx " << t << " has not been submitted.");
		}
		if (!c->gridSet) USGB_FAIL(USGB_ERR_INVALID_STATE, "The grid has not been set.");
		if (c->hOutCap < 2 * static_cast<size_t>(c->npix)) {
			if (c->h_out) { cudaFreeHost(c->h_out); c->h_out = nullptr; c->hOutCap = 0; }
			USGB_CUDA(cudaMallocHost(&c->h_out, 2 * static_cast<size_t>(c->npix) * sizeof(float)));
			c->hOutCap = 2 * static_cast<size_t>(c->npix);
		}
		run_frame(c, c->d_rf, c->d_value, c->d_factor);  // the RF transfers were queued by usgb_submit_rf
		USGB_CUDA(cudaMemcpyAsync(c->h_out, c->d_value, c->npix * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
		USGB_CUDA(cudaMemcpyAsync(c->h_out + c->npix, c->d_factor, c->npix * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
		USGB_CUDA(cudaStreamSynchronize(c->stream));
		unsigned errWord = 0;
		USGB_CUDA(cudaMemcpy(&errWord, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
		if (errWord) USGB_FAIL(USGB_ERR_DEVICE_TIMEOUT, "device-side wait gave up (code " << errWord << ")");
		std::memcpy(value, c->h_out, c->npix * sizeof(float));
		if (factor) std::memcpy(factor, c->h_out + c->npix, c->npix * sizeof(float));
	});
}

int usgb_process_rf(usgb_ctx* c, const float* rf, float* value, float* factor)
{
	return guarded(c, [&] {
		if (!rf || !value) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "null host pointer");
		if (!c->gridSet) USGB_FAIL(USGB_ERR_INVALID_STATE, "The grid has not been set.");
		if (c->hostDirect) {
			// The preparation kernel reads the RF and the delay-and-sum writes
			// the images in host memory, through the host's page tables.
			run_frame(c, rf, value, factor ? factor : c->d_factor);
		} else {
			const size_t rfBytes = static_cast<size_t>(c->numSignals) * c->prm.num_samples * sizeof(float);
			USGB_CUDA(cudaMemcpyAsync(c->d_rf, rf, rfBytes, cudaMemcpyHostToDevice, c->stream));
			run_frame(c, c->d_rf, c->d_value, c->d_factor);
			USGB_CUDA(cudaMemcpyAsync(value, c->d_value, c->npix * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
			if (factor) {
				USGB_CUDA(cudaMemcpyAsync(factor, c->d_factor, c->npix * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
			}
		}
		USGB_CUDA(cudaStreamSynchronize(c->stream));
		unsigned errWord = 0;
		USGB_CUDA(cudaMemcpy(&errWord, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
		if (errWord) USGB_FAIL(USGB_ERR_DEVICE_TIMEOUT, "device-side wait gave up (code " << errWord << ")");
	});
}

int usgb_set_wait_test(usgb_ctx* c, uint32_t wait_limit_us, uint32_t skip_stage)
{
	return guarded(c, [&] {
		c->waitLimitNs = static_cast<unsigned long long>(wait_limit_us) * 1000ull;
		c->testSkipStage = skip_stage;
	});
}

int usgb_set_host_direct(usgb_ctx* c, int enable)
{
	return guarded(c, [&] {
		if (enable && !c->hostDirectAvailable) {
			USGB_FAIL(USGB_ERR_UNSUPPORTED, "This device cannot access pageable host memory through the host's page tables.");
		}
		c->hostDirect = enable != 0;
	});
}

int usgb_get_host_direct(const usgb_ctx* c, int* available, int* enabled)
{
	if (!c) return USGB_ERR_INVALID_PARAMETER;
	if (available) *available = c->hostDirectAvailable ? 1 : 0;
	if (enabled) *enabled = c->hostDirect ? 1 : 0;
	return USGB_OK;
}

int usgb_process_device(usgb_ctx* c, const float* d_rf, float* d_value, float* d_factor)
{
	return guarded(c, [&] {
		if (!d_rf || !d_value || !d_factor) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "null device pointer");
		run_frame(c, d_rf, d_value, d_factor);
	});
}

int usgb_prepare_signals_device(usgb_ctx* c, const float* d_rf, void* d_signals)
{
	return guarded(c, [&] {
		if (!d_rf || !d_signals) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "null device pointer");
		if (reinterpret_cast<uintptr_t>(d_signals) % 16 != 0) {
			USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "The signal tensor must be 16-byte aligned.");
		}
		const usgb::PrepParams pp = prep_params(c, d_rf, d_signals);
		USGB_CUDA(usgb::launch_prep(pp, static_cast<int>(c->prm.storage), c->analytic, c->stream));
	});
}

int usgb_delay_and_sum_device(usgb_ctx* c, const void* d_signals, float* d_value, float* d_factor)
{
	return guarded(c, [&] {
		if (!d_signals || !d_value || !d_factor) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "null device pointer");
		if (!c->gridSet) USGB_FAIL(USGB_ERR_INVALID_STATE, "The grid has not been set.");
		if (reinterpret_cast<uintptr_t>(d_signals) % 16 != 0) {
			USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "The signal tensor must be 16-byte aligned.");
		}
		USGB_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
		const usgb::DasParams dp = das_params(c, d_signals, d_value, d_factor);
		USGB_CUDA(usgb::launch_das(dp, static_cast<int>(c->prm.storage), static_cast<int>(c->prm.coherence),
				c->analytic, c->dasVariant, c->stream));
	});
}

int usgb_signal_info(const usgb_ctx* c, uint32_t* signal_length, uint32_t* fft_size, uint32_t* signal_stride, size_t* signal_bytes)
{
	if (!c) return USGB_ERR_INVALID_PARAMETER;
	if (signal_length) *signal_length = c->L;
	if (fft_size) *fft_size = c->fft.N;
	if (signal_stride) *signal_stride = c->sigStride;
	if (signal_bytes) *signal_bytes = c->sigBytes;
	return USGB_OK;
}

int usgb_set_das_variant(usgb_ctx* c, int variant, uint32_t tile_rows, uint32_t stage_bytes, uint32_t stages)
{
	return guarded(c, [&] {
		if (variant < 0 || variant > 4) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid delay-and-sum variant: " << variant << '.');
		const unsigned rows = tile_rows ? tile_rows : c->tileRows;
		const unsigned cap = stage_bytes ? stage_bytes : c->stageBytes;
		const unsigned nst = stages ? stages : c->stages;
		if (variant != 0) {
			if (variant >= 3) {
				if (rows < 1 || rows > 8) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "64-column tiles have 1 to 8 rows.");
			} else if (rows != 4 && rows != 8 && rows != 16) {
				USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Tile rows must be 4, 8 or 16.");
			}
			if (cap < 1024 || cap % 128 != 0 || cap > (1u << 20)) {
				USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Stage size must be a multiple of 128 bytes in [1 KiB, 1 MiB].");
			}
			if (nst < 2 || nst > 16) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Stage count must be in [2, 16].");
			const size_t need = das_smem_bytes(c, variant, rows, cap, nst);
			if (need > max_smem()) {
				USGB_FAIL(USGB_ERR_UNSUPPORTED, "Staged delay-and-sum needs " << need << " bytes of shared memory (device: "
						<< max_smem() << "); use fewer tile rows, stages or smaller stages.");
			}
		}
		c->dasVariant = variant;
		c->tileRows = rows;
		c->stageBytes = cap;
		c->stages = nst;
		c->dasExplicit = true;
	});
}

int usgb_set_delay_precision(usgb_ctx* c, uint32_t mode)
{
	return guarded(c, [&] {
		if (mode > USGB_DELAY_FP64) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid delay precision: " << mode << '.');
		c->delayMode = static_cast<int>(mode);
	});
}

int usgb_get_das_config(const usgb_ctx* c, int* variant, uint32_t* tile_rows, uint32_t* stage_bytes, uint32_t* stages)
{
	if (!c) return USGB_ERR_INVALID_PARAMETER;
	if (variant) *variant = c->dasVariant;
	if (tile_rows) *tile_rows = c->tileRows;
	if (stage_bytes) *stage_bytes = c->stageBytes;
	if (stages) *stages = c->stages;
	return USGB_OK;
}

int usgb_autotune_das(usgb_ctx* c, const void* d_signals, float* d_value, float* d_factor, uint32_t iterations,
		float* best_ms)
{
	return guarded(c, [&] {
		if (!d_signals || !d_value || !d_factor) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "null device pointer");
		if (!c->gridSet) USGB_FAIL(USGB_ERR_INVALID_STATE, "The grid has not been set.");
		if (reinterpret_cast<uintptr_t>(d_signals) % 16 != 0) {
			USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "The signal tensor must be 16-byte aligned.");
		}
		const unsigned iters = iterations ? iterations : 3;
		struct Cand { int variant; unsigned rows, cap, stages; };
		std::vector<Cand> cands;
		for (int variant : {1, 2, 3, 4})
			for (unsigned rows : {4u, 5u, 6u, 7u, 8u, 16u})
				for (unsigned cap : {8192u, 12288u, 16384u, 20480u, 24576u, 32768u, 49152u, 65536u, 98304u, 102400u,
						110592u})
					for (unsigned nst : {2u, 3u, 4u})
						if ((variant >= 2 || cap % 8192u == 0) && !(variant >= 3 && rows == 16)
								&& (variant >= 3 || rows == 4 || rows == 8 || rows == 16)
								&& das_smem_bytes(c, variant, rows, cap, nst) <= max_smem())
							cands.push_back({variant, rows, cap, nst});
		cands.push_back({0, c->tileRows, c->stageBytes, c->stages});
		cudaEvent_t e0, e1;
		USGB_CUDA(cudaEventCreate(&e0));
		USGB_CUDA(cudaEventCreate(&e1));
		float best = 1e30f;
		Cand bestC = cands.back();
		const Cand saved{c->dasVariant, c->tileRows, c->stageBytes, c->stages};
		for (const Cand& k : cands) {
			c->dasVariant = k.variant;
			c->tileRows = k.rows;
			c->stageBytes = k.cap;
			c->stages = k.stages;
			const usgb::DasParams dp = das_params(c, d_signals, d_value, d_factor);
			USGB_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
			USGB_CUDA(usgb::launch_das(dp, static_cast<int>(c->prm.storage), static_cast<int>(c->prm.coherence),
					c->analytic, k.variant, c->stream));  // warm-up
			USGB_CUDA(cudaEventRecord(e0, c->stream));
			for (unsigned i = 0; i < iters; ++i) {
				USGB_CUDA(usgb::launch_das(dp, static_cast<int>(c->prm.storage), static_cast<int>(c->prm.coherence),
						c->analytic, k.variant, c->stream));
			}
			USGB_CUDA(cudaEventRecord(e1, c->stream));
			USGB_CUDA(cudaEventSynchronize(e1));
			unsigned errWord = 0;
			USGB_CUDA(cudaMemcpy(&errWord, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
			float ms = 0;
			USGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
			ms /= static_cast<float>(iters);
			if (!errWord && ms < best) {
				best = ms;
				bestC = k;
			}
		}
		cudaEventDestroy(e0);
		cudaEventDestroy(e1);
		if (best >= 1e30f) {
			c->dasVariant = saved.variant;
			c->tileRows = saved.rows;
			c->stageBytes = saved.cap;
			c->stages = saved.stages;
			USGB_FAIL(USGB_ERR_DEVICE_TIMEOUT, "no delay-and-sum configuration completed");
		}
		c->dasVariant = bestC.variant;
		c->tileRows = bestC.rows;
		c->stageBytes = bestC.cap;
		c->stages = bestC.stages;
		c->dasExplicit = true;
		if (best_ms) *best_ms = best;
	});
}

int usgb_synchronize(usgb_ctx* c)
{
	return guarded(c, [&] {
		USGB_CUDA(cudaStreamSynchronize(c->stream));
		unsigned errWord = 0;
		USGB_CUDA(cudaMemcpy(&errWord, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
		if (errWord) USGB_FAIL(USGB_ERR_DEVICE_TIMEOUT, "device-side wait gave up (code " << errWord << ")");
	});
}

}  // extern "C"

// ===========================================================================
// Batched frames
// ===========================================================================
namespace {

size_t batch_desc_bytes(unsigned maxFrames)
{
	return sizeof(usgb::BatchHeader) + maxFrames * (sizeof(usgb::BatchPrepFrame) + sizeof(usgb::BatchDasFrame));
}

// Largest prep shared memory over the batch's frames.
size_t batch_prep_smem(const usgb_batch_item* items, uint32_t count)
{
	size_t m = 0;
	for (uint32_t i = 0; i < count; ++i) {
		const usgb::PrepParams pp = prep_params(items[i].ctx, nullptr, nullptr);
		m = std::max(m, usgb::prep_smem_bytes(pp, items[i].ctx->analytic));
	}
	return m;
}

template<typename F>
int batch_guarded(usgb_batch* b, F&& f)
{
	if (!b) return USGB_ERR_INVALID_PARAMETER;
	try {
		f();
		return USGB_OK;
	} catch (const Failure& e) {
		b->err = e.msg;
		return e.code;
	} catch (const std::exception& e) {
		b->err = e.what();
		return USGB_ERR_INVALID_STATE;
	}
}

size_t batch_das_smem(const usgb_batch* b, int variant, unsigned rows, unsigned cap, unsigned nst)
{
	return variant >= 2 ? usgb::das_group_smem_bytes(b->maxElements, b->maxElements, usgb::das_tile_cols(variant), rows, cap, nst)
	                    : usgb::das_staged_smem_bytes(b->maxElements, b->maxElements, rows, cap, nst);
}

}  // namespace

extern "C" {

int usgb_batch_create(uint32_t max_frames, uint32_t max_elements, uint32_t max_signal_length, usgb_batch** out)
{
	if (!out) return USGB_ERR_INVALID_PARAMETER;
	*out = nullptr;
	usgb_batch* b = nullptr;
	try {
		if (max_frames == 0 || max_frames > 4096) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "max_frames must be in [1, 4096].");
		if (max_elements == 0 || max_elements > 1024) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "max_elements must be in [1, 1024].");
		b = new usgb_batch();
		b->maxFrames = max_frames;
		b->maxElements = max_elements;
		b->maxSignalLength = max_signal_length;
		int dev = 0, sms = 0;
		USGB_CUDA(cudaGetDevice(&dev));
		USGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
		b->numSMs = static_cast<unsigned>(sms);
		if (batch_das_smem(b, b->dasVariant, b->tileRows, b->stageBytes, b->stages) > max_smem()) {
			b->stageBytes = 8192;
			if (batch_das_smem(b, b->dasVariant, b->tileRows, b->stageBytes, b->stages) > max_smem()) {
				USGB_FAIL(USGB_ERR_UNSUPPORTED, "max_elements too large for the batched delay-and-sum.");
			}
		}
		b->descBytes = batch_desc_bytes(max_frames);
		USGB_CUDA(cudaMallocHost(&b->h_desc, b->descBytes));
		USGB_CUDA(cudaMalloc(&b->d_desc, b->descBytes));
		USGB_CUDA(cudaMalloc(&b->d_err, sizeof(unsigned)));
		USGB_CUDA(cudaMemset(b->d_err, 0, sizeof(unsigned)));
		USGB_CUDA(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
		*out = b;
		return USGB_OK;
	} catch (const Failure& e) {
		g_createError = e.msg;
		delete b;
		return e.code;
	}
}

void usgb_batch_destroy(usgb_batch* b)
{
	if (!b) return;
	if (b->pending) cudaEventSynchronize(b->done);
	delete b;
}

const char* usgb_batch_last_error(const usgb_batch* b)
{
	return b ? b->err.c_str() : g_createError.c_str();
}

int usgb_batch_set_das_variant(usgb_batch* b, int variant)
{
	return batch_guarded(b, [&] {
		if (variant < 1 || variant > 4) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Batched delay-and-sum variant must be 1, 2, 3 or 4.");
		if (variant >= 3 && b->tileRows == 16) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "64-column tiles have 4 or 8 rows.");
		if (variant != 4 && b->tileRows == 7) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "7 tile rows need two points per thread (variant 4).");
		if (batch_das_smem(b, variant, b->tileRows, b->stageBytes, b->stages) > max_smem()) {
			USGB_FAIL(USGB_ERR_UNSUPPORTED, "the current tile shape does not fit in shared memory for this variant.");
		}
		b->dasVariant = variant;
		if (b->graph) {
			cudaGraphExecDestroy(b->graph);
			b->graph = nullptr;
		}
	});
}

int usgb_batch_set_das_config(usgb_batch* b, uint32_t tile_rows, uint32_t stage_bytes, uint32_t stages)
{
	return batch_guarded(b, [&] {
		if (tile_rows != 4 && tile_rows != 8 && tile_rows != 16 && !(tile_rows == 7 && b->dasVariant == 4)) {
			USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Tile rows must be 4, 8 or 16 (or 7 with two points per thread).");
		}
		if (b->dasVariant >= 3 && tile_rows == 16) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "64-column tiles have 4 or 8 rows.");
		if (stage_bytes < 1024 || stage_bytes % 128 != 0 || stage_bytes > (1u << 20)) {
			USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Stage size must be a multiple of 128 bytes in [1 KiB, 1 MiB].");
		}
		if (stages < 2 || stages > 16) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Stage count must be in [2, 16].");
		if (batch_das_smem(b, b->dasVariant, tile_rows, stage_bytes, stages) > max_smem()) {
			USGB_FAIL(USGB_ERR_UNSUPPORTED, "configuration does not fit in shared memory for max_elements "
					<< b->maxElements << '.');
		}
		b->tileRows = tile_rows;
		b->stageBytes = stage_bytes;
		b->stages = stages;
		if (b->graph) {
			cudaGraphExecDestroy(b->graph);
			b->graph = nullptr;
		}
	});
}

int usgb_batch_run(usgb_batch* b, const usgb_batch_item* items, uint32_t count, void* cuda_stream, int use_graph)
{
	return batch_guarded(b, [&] {
		if (!items || count == 0) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "empty batch");
		if (count > b->maxFrames) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Batch of " << count << " frames exceeds max_frames "
				<< b->maxFrames << '.');
		cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);
		const usgb_ctx* c0 = items[0].ctx;
		if (!c0) USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "null context in batch");
		for (uint32_t i = 0; i < count; ++i) {
			const usgb_ctx* c = items[i].ctx;
			if (!c || !items[i].d_rf || !items[i].d_value || !items[i].d_factor) {
				USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "null pointer in batch item " << i << '.');
			}
			if (c->prm.storage != c0->prm.storage || c->analytic != c0->analytic) {
				USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "All frames of a batch share the storage type and signal path.");
			}
			if (!c->gridSet) USGB_FAIL(USGB_ERR_INVALID_STATE, "The grid of batch item " << i << " has not been set.");
			if (c->prm.num_tx > b->maxElements || c->prm.num_rx > b->maxElements) {
				USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Batch item " << i << " has more elements than max_elements.");
			}
			if (b->maxSignalLength && c->L > b->maxSignalLength) {
				USGB_FAIL(USGB_ERR_INVALID_PARAMETER, "Batch item " << i << " exceeds max_signal_length.");
			}
		}
		// The descriptor buffer of the previous run must have been consumed.
		if (b->pending) {
			USGB_CUDA(cudaEventSynchronize(b->done));
			b->pending = false;
		}
		auto* hdr = reinterpret_cast<usgb::BatchHeader*>(b->h_desc);
		auto* prepF = reinterpret_cast<usgb::BatchPrepFrame*>(b->h_desc + sizeof(usgb::BatchHeader));
		auto* dasF = reinterpret_cast<usgb::BatchDasFrame*>(b->h_desc + sizeof(usgb::BatchHeader)
				+ b->maxFrames * sizeof(usgb::BatchPrepFrame));
		unsigned sigBegin = 0, tileBegin = 0;
		for (uint32_t i = 0; i < count; ++i) {
			usgb_ctx* c = items[i].ctx;
			prepF[i].prep = prep_params(c, items[i].d_rf, c->d_sig);
			prepF[i].signalBegin = sigBegin;
			sigBegin += c->numSignals;
			usgb::DasParams dp = das_params(c, c->d_sig, items[i].d_value, items[i].d_factor);
			dp.errWord = b->d_err;
			dp.tileCols = usgb::das_tile_cols(b->dasVariant);
			dp.tileRows = b->tileRows;
			dp.stageBytes = b->stageBytes;
			dp.stages = b->stages;
			dp.pointsPerThread = usgb::das_points_per_thread(b->dasVariant);
			dasF[i].das = dp;
			dasF[i].tileBegin = tileBegin;
			dasF[i].tilesX = (c->ncols + dp.tileCols - 1) / dp.tileCols;
			dasF[i].cf = static_cast<int>(c->prm.coherence);
			const unsigned tileH = b->tileRows * dp.pointsPerThread;
			tileBegin += dasF[i].tilesX * ((c->nrows + tileH - 1) / tileH);
		}
		hdr->count = count;
		hdr->totalSignals = sigBegin;
		hdr->totalTiles = tileBegin;
		const auto* dHdr = reinterpret_cast<const usgb::BatchHeader*>(b->d_desc);
		const auto* dPrep = reinterpret_cast<const usgb::BatchPrepFrame*>(b->d_desc + sizeof(usgb::BatchHeader));
		const auto* dDas = reinterpret_cast<const usgb::BatchDasFrame*>(b->d_desc + sizeof(usgb::BatchHeader)
				+ b->maxFrames * sizeof(usgb::BatchPrepFrame));
		const size_t prepSmem = batch_prep_smem(items, count);
		if (prepSmem > max_smem()) USGB_FAIL(USGB_ERR_UNSUPPORTED, "An A-scan of the batch is too long for on-chip preparation.");
		unsigned maxL = 0;
		for (uint32_t i = 0; i < count; ++i) maxL = std::max(maxL, items[i].ctx->L);
		const unsigned tmemCols = usgb::prep_batch_tmem_columns(prepSmem, maxL, items[0].ctx->analytic);
		for (uint32_t i = 0; i < count; ++i) prepF[i].prep.tmemCols = tmemCols;
		const unsigned prepPerSM = std::max<unsigned>(1, static_cast<unsigned>((228u * 1024u) / (prepSmem + 1024u)));
		const unsigned prepBlocks = b->numSMs * std::min(prepPerSM, 4u);
		usgb::BatchDasConfig dc{};
		dc.maxTx = dc.maxRx = b->maxElements;
		dc.tileCols = usgb::das_tile_cols(b->dasVariant);
		dc.tileRows = b->tileRows;
		dc.stageBytes = b->stageBytes;
		dc.stages = b->stages;
		dc.pointsPerThread = usgb::das_points_per_thread(b->dasVariant);
		if (b->dasVariant >= 2) {
			dc.blocks = 0;  // the launcher fills the SMs (occupancy of the kernel at this shape)
		} else {
			const size_t dasSmem = usgb::das_staged_smem_bytes(dc.maxTx, dc.maxRx, dc.tileRows, dc.stageBytes, dc.stages);
			const unsigned dasPerSM = std::max<unsigned>(1, static_cast<unsigned>((228u * 1024u) / (dasSmem + 1024u)));
			dc.blocks = b->numSMs * std::min(dasPerSM, 4u);
		}
		const int variant = b->dasVariant;
		const int storage = static_cast<int>(c0->prm.storage);
		const bool analytic = c0->analytic;

		auto enqueue = [&](cudaStream_t st) {
			USGB_CUDA(cudaMemcpyAsync(b->d_desc, b->h_desc, b->descBytes, cudaMemcpyHostToDevice, st));
			USGB_CUDA(usgb::launch_prep_batch(dPrep, dHdr, prepSmem, prepBlocks, storage, analytic, st));
			if (variant >= 2) {
				USGB_CUDA(usgb::launch_das_group_batch(dDas, dHdr, dc, storage, analytic, st));
			} else {
				USGB_CUDA(usgb::launch_das_staged_batch(dDas, dHdr, dc, storage, analytic, st));
			}
		};
		if (use_graph) {
			// Re-capture when the launch shape changed (the kernels read the
			// frames from the descriptor buffer, so the graph is frame-agnostic).
			if (!b->graph || b->graphPrepSmem < prepSmem || b->graphStorage != storage || b->graphAnalytic != analytic) {
				if (b->graph) {
					cudaGraphExecDestroy(b->graph);
					b->graph = nullptr;
				}
				cudaStream_t cap;
				USGB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
				cudaGraph_t g = nullptr;
				USGB_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
				try {
					enqueue(cap);
				} catch (...) {
					cudaStreamEndCapture(cap, &g);
					if (g) cudaGraphDestroy(g);
					cudaStreamDestroy(cap);
					throw;
				}
				USGB_CUDA(cudaStreamEndCapture(cap, &g));
				const cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
				cudaGraphDestroy(g);
				cudaStreamDestroy(cap);
				USGB_CUDA(ie);
				b->graphPrepSmem = prepSmem;
				b->graphStorage = storage;
				b->graphAnalytic = analytic;
			}
			USGB_CUDA(cudaGraphLaunch(b->graph, stream));
		} else {
			enqueue(stream);
		}
		USGB_CUDA(cudaEventRecord(b->done, stream));
		b->pending = true;
	});
}

int usgb_batch_synchronize(usgb_batch* b)
{
	return batch_guarded(b, [&] {
		if (b->pending) {
			USGB_CUDA(cudaEventSynchronize(b->done));
			b->pending = false;
		}
		unsigned errWord = 0;
		USGB_CUDA(cudaMemcpy(&errWord, b->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
		if (errWord) {
			USGB_CUDA(cudaMemset(b->d_err, 0, sizeof(unsigned)));
			USGB_FAIL(USGB_ERR_DEVICE_TIMEOUT, "device-side wait gave up (code " << errWord << ")");
		}
	});
}

}  // extern "C"
