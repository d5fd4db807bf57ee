// Frame parameter checks and the constants derived from them, shared by every
// entry point that takes a usgb_sta_params (usgb_create in usgb_api.cu and the
// allocation-free usgb_process_frame_noalloc in usgb_noalloc.cu), so that the
// two apply the same rules with the same messages. Host code only.
//
// Rules and messages follow the reference's processor constructors and
// STAConfiguration::load ranges (src/user/configuration/STAConfiguration.h:55-75,
// src/user/processor/VectorialSTAProcessor.h:120-160, CoherenceFactor.h:63-76,
// 139-152): dead zone, upsampling, coherence-factor parameters.
#pragma once

#include <cmath>
#include <cstdint>
#include <limits>
#include <sstream>
#include <string>

#include "../../include/usgb.h"
#include "usgb_tables.h"

namespace usgb {
namespace host {

// A rejected parameter: the status code and the message.
struct ParamError {
	int code;
	std::string msg;
};

#define USGB_PARAM_FAIL(CODE, STREAM_EXPR)          \
	do {                                            \
		std::ostringstream os_;                     \
		os_ << STREAM_EXPR;                         \
		throw ::usgb::host::ParamError{(CODE), os_.str()}; \
	} while (0)

// Constants of one frame, derived from checked parameters.
struct FrameConsts {
	bool analytic;
	unsigned U;            // upsampling factor
	unsigned L;            // signal length after upsampling
	unsigned numSignals;   // num_tx * num_rx A-scans
	unsigned deadZone;     // deadZoneSamplesUp_ (VectorialSTAProcessor.h:138)
	unsigned sigStride;    // samples per A-scan in the signal tensor (L rounded up to 8)
	size_t elemBytes;      // bytes per stored sample (complex or real, FP32 or 16-bit)
	float invCT;           // fs * U / c (VectorialSTAProcessor.h:241)
	float signalOffset;    // fs * U * peakOffset / fc (VectorialSTAProcessor.h:147)
	float valueCoef;       // 1 / (num_tx * num_rx) (VectorialSTAProcessor.h:337-338)
	float pcfFactor;       // gamma / sigma0, sigma0 = pi / sqrt(3) (CoherenceFactor.h:288-296)
	float scale;           // storage scale (1 for FP32 or when 0)
};

// Throws ParamError when a parameter is out of range.
inline FrameConsts check_frame_params(const usgb_sta_params* p)
{
	if (!p) USGB_PARAM_FAIL(USGB_ERR_INVALID_PARAMETER, "null parameters");
	if (p->num_tx == 0 || p->num_rx == 0) USGB_PARAM_FAIL(USGB_ERR_INVALID_PARAMETER, "The number of elements is zero.");
	if (p->num_tx > 1024 || p->num_rx > 1024) USGB_PARAM_FAIL(USGB_ERR_INVALID_PARAMETER, "More than 1024 elements.");
	if (p->num_samples == 0) USGB_PARAM_FAIL(USGB_ERR_INVALID_PARAMETER, "The number of samples is zero.");
	if (!p->tx_xy || !p->rx_xy) USGB_PARAM_FAIL(USGB_ERR_INVALID_PARAMETER, "Missing element positions.");
	if (p->signal_path != USGB_PATH_ANALYTIC && p->signal_path != USGB_PATH_REAL) {
		USGB_PARAM_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid signal path: " << p->signal_path << '.');
	}
	FrameConsts c{};
	c.analytic = p->signal_path == USGB_PATH_ANALYTIC;
	if (c.analytic) {
		if (p->upsampling == 0 || p->upsampling > 64) {
			USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "Invalid upsampling factor: " << p->upsampling << ". Must be >= 1 and <= 64.");
		}
	} else if (p->upsampling != 4) {
		USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "The real-RF path upsamples by 4 (got " << p->upsampling << ").");
	}
	if (!(p->sampling_frequency > 0) || !(p->propagation_speed > 0) || !(p->center_frequency > 0)) {
		USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "Sampling frequency, propagation speed and center frequency must be > 0.");
	}
	if (!(p->dead_zone_m >= 0)) USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "Invalid dead zone: " << p->dead_zone_m << '.');
	if (p->coherence > USGB_CF_MF) {
		USGB_PARAM_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid coherence factor method: " << p->coherence << '.');
	}
	if (!c.analytic && p->coherence != USGB_CF_NONE && p->coherence != USGB_CF_SCF) {
		USGB_PARAM_FAIL(USGB_ERR_INVALID_PARAMETER, "The real-RF path supports only the sign coherence factor.");
	}
	if (p->coherence == USGB_CF_PCF && !(p->pcf_gamma >= 0 && p->pcf_gamma <= 100)) {
		USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "Invalid phase_coherence_factor_gamma: " << p->pcf_gamma << '.');
	}
	if (p->coherence == USGB_CF_SCF && !(p->scf_p >= 0 && p->scf_p <= 100)) {
		USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "Invalid sign_coherence_factor_p: " << p->scf_p << '.');
	}
	if (p->storage > USGB_STORE_BF16) USGB_PARAM_FAIL(USGB_ERR_INVALID_PARAMETER, "Invalid storage type: " << p->storage << '.');

	c.U = p->upsampling;
	c.numSignals = p->num_tx * p->num_rx;
	const unsigned long long L = static_cast<unsigned long long>(p->num_samples) * c.U;
	if (L < 2) USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "The signal length (" << L << ") must be >= 2.");
	if (c.analytic && L > (1ULL << 20)) {
		USGB_PARAM_FAIL(USGB_ERR_INVALID_PARAMETER, "The number of input samples (" << L << ") is greater than " << (1U << 20) << '.');
	}
	c.L = static_cast<unsigned>(L);
	const float upFs = c.U * p->sampling_frequency;
	const double dz = upFs * 2.0 * p->dead_zone_m / p->propagation_speed;
	if (!(dz < static_cast<double>(std::numeric_limits<unsigned>::max()))) {
		USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "Invalid dead zone: " << p->dead_zone_m << '.');
	}
	c.deadZone = static_cast<unsigned>(dz);
	if (c.deadZone >= c.L) {
		USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "Invalid dead zone: deadZoneSamplesUp_ (" << c.deadZone
				<< ") >= signalLength (" << c.L << ").");
	}
	c.invCT = upFs / p->propagation_speed;
	c.signalOffset = upFs * p->peak_offset / p->center_frequency;
	c.valueCoef = 1.0f / static_cast<float>(c.numSignals);
	c.pcfFactor = p->pcf_gamma / static_cast<float>(kPi / std::sqrt(3.0));
	c.scale = (p->storage == USGB_STORE_F32 || p->storage_scale == 0.0f) ? 1.0f : p->storage_scale;
	c.elemBytes = (c.analytic ? 2 : 1) * (p->storage == USGB_STORE_F32 ? 4 : 2);
	c.sigStride = (c.L + 7U) & ~7U;
	return c;
}

// Grid size checks (the reference's "Zero columns/rows" messages); returns
// the number of grid points, at most 2^31.
inline size_t check_grid_size(uint32_t ncols, uint32_t nrows)
{
	if (ncols == 0) USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "Zero columns in the grid.");
	if (nrows == 0) USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "Zero rows in the grid.");
	const size_t npix = static_cast<size_t>(ncols) * nrows;
	if (npix > (1ULL << 31)) USGB_PARAM_FAIL(USGB_ERR_INVALID_VALUE, "Grid too large.");
	return npix;
}

}  // namespace host
}  // namespace usgb
