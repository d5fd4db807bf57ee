// Drop-in processor classes for the reference tree (us_lab4a), built on the C
// ABI of usgb.h. Header-only; include it from a translation unit that sees the
// reference's headers (ArrayProcessor.h, STAConfiguration.h, SA3DConfiguration.h,
// STAAcquisition.h, CoherenceFactor.h, ArrayGeometry.h, Exception.h) and link
// libusgb.so.
//
//   VectorialSTAGB300Processor   same constructor as VectorialSTACUDAProcessor
//                                (src/user/processor/VectorialSTACUDAProcessor.h:65-71)
//   Vectorial3DSTAGB300Processor same constructor as Vectorial3DSTAProcessor<float>
//                                (src/user/processor/Vectorial3DSTAProcessor.h:54-60)
//   DefaultSTAGB300Processor     same constructor as DefaultSTAProcessor<float, XYZValueFactor<float>>
//                                (src/user/processor/DefaultSTAProcessor.h:54-58)
//
// Lifecycle mirrors the reference: the signal length is taken from the first
// acquisition in process() (lazy initialisation); the A-scans of every
// transmit event are handed to the library, the image is formed on the GPU,
// and value / factor are written back into gridData. Library status codes are
// rethrown as the reference's exception types.
#ifndef USGB_STA_PROCESSOR_HPP
#define USGB_STA_PROCESSOR_HPP

#include <string>
#include <vector>

#include "usgb.h"

namespace Lab {

namespace usgb_detail {

inline void check(int rc, const usgb_ctx* ctx)
{
	if (rc == USGB_OK) return;
	const std::string msg = usgb_last_error(ctx);
	switch (rc) {
	case USGB_ERR_INVALID_PARAMETER: THROW_EXCEPTION(InvalidParameterException, msg);
	case USGB_ERR_INVALID_VALUE: THROW_EXCEPTION(InvalidValueException, msg);
	case USGB_ERR_INVALID_STATE: THROW_EXCEPTION(InvalidStateException, msg);
	default: THROW_EXCEPTION(Exception, "[usgb " << rc << "] " << msg);
	}
}

// Runs one frame: RF of every transmit event from the acquisition, grid
// coordinates from gridData, value/factor back into gridData.
template<typename Acquisition>
void run_frame(usgb_ctx*& ctx, usgb_sta_params& params, std::vector<float>& txXY, std::vector<float>& rxXY,
		const std::vector<float>& apod, Acquisition& acquisition, const std::vector<unsigned int>& txElems,
		Matrix<XYZValueFactor<float>>& gridData, std::vector<float>& xyz, std::vector<float>& value,
		std::vector<float>& factor)
{
	Util::resetValueFactor(gridData.begin(), gridData.end());
	if (gridData.n1() == 0) THROW_EXCEPTION(InvalidValueException, "Zero columns in the grid.");
	typename STAAcquisition<float>::AcquisitionDataType acqData;
	for (std::size_t i = 0; i < txElems.size(); ++i) {
		acquisition.execute(txElems[i], acqData);
		if (!ctx) {
			params.num_samples = static_cast<uint32_t>(acqData.n2());
			params.tx_xy = txXY.data();
			params.rx_xy = rxXY.data();
			params.rx_apod = apod.empty() ? nullptr : apod.data();
			check(usgb_create(&params, &ctx), nullptr);
		}
		check(usgb_submit_rf(ctx, static_cast<uint32_t>(i), &acqData(0, 0),
				static_cast<uint32_t>(acqData.n1()), static_cast<uint32_t>(acqData.n2())), ctx);
	}
	const std::size_t n = gridData.size();
	xyz.resize(3 * n);
	for (std::size_t p = 0; p < n; ++p) {
		const XYZValueFactor<float>& point = *(gridData.data() + p);
		xyz[3 * p] = point.x;
		xyz[3 * p + 1] = point.y;
		xyz[3 * p + 2] = point.z;
	}
	check(usgb_set_grid(ctx, xyz.data(), static_cast<uint32_t>(gridData.n1()), static_cast<uint32_t>(gridData.n2())), ctx);
	value.resize(n);
	factor.resize(n);
	check(usgb_process(ctx, value.data(), factor.data()), ctx);
	for (std::size_t p = 0; p < n; ++p) {
		XYZValueFactor<float>& point = *(gridData.data() + p);
		point.value = value[p];
		point.factor = factor[p];
	}
}

inline uint32_t analytic_cf(const AnalyticSignalCoherenceFactorProcessor<float>& cf, float& gamma)
{
	if (!cf.enabled()) return USGB_CF_NONE;
	std::vector<float> constants;
	cf.implementation().getConstants(constants);  // {gamma, sigma0, gamma / sigma0}
	gamma = constants.at(0);
	return USGB_CF_PCF;
}

}  // namespace usgb_detail

class VectorialSTAGB300Processor : public ArrayProcessor<XYZValueFactor<float>> {
public:
	VectorialSTAGB300Processor(const STAConfiguration<float>& config, STAAcquisition<float>& acquisition,
			unsigned int upsamplingFactor, AnalyticSignalCoherenceFactorProcessor<float>& coherenceFactor,
			float peakOffset, const std::vector<float>& rxApod, uint32_t storage = USGB_STORE_F32)
		: config_(config), acquisition_(acquisition), rxApod_(rxApod), params_()
	{
		std::vector<float> x;
		ArrayGeometry::getElementXCentered2D(config_.numElements, config_.pitch, x);
		for (unsigned e = 0; e < config_.numElements; ++e) {
			rxXY_.push_back(x[e]);
			rxXY_.push_back(0.0f);
		}
		for (unsigned e = config_.firstTxElem; e <= config_.lastTxElem; ++e) {
			txXY_.push_back(x[e]);
			txXY_.push_back(0.0f);
			txElems_.push_back(e);
		}
		params_.num_tx = static_cast<uint32_t>(txElems_.size());
		params_.num_rx = config_.numElements;
		params_.upsampling = upsamplingFactor;
		params_.signal_path = USGB_PATH_ANALYTIC;
		params_.sampling_frequency = config_.samplingFrequency;
		params_.propagation_speed = config_.propagationSpeed;
		params_.center_frequency = config_.centerFrequency;
		params_.peak_offset = peakOffset;
		params_.dead_zone_m = config_.deadZoneM;
		params_.coherence = usgb_detail::analytic_cf(coherenceFactor, params_.pcf_gamma);
		params_.storage = storage;
	}
	virtual ~VectorialSTAGB300Processor() { usgb_destroy(ctx_); }

	virtual void prepare(unsigned int baseElement) { acquisition_.prepare(baseElement); }
	virtual void process(Matrix<XYZValueFactor<float>>& gridData)
	{
		usgb_detail::run_frame(ctx_, params_, txXY_, rxXY_, rxApod_, acquisition_, txElems_, gridData, xyz_,
				value_, factor_);
	}
private:
	VectorialSTAGB300Processor(const VectorialSTAGB300Processor&) = delete;
	VectorialSTAGB300Processor& operator=(const VectorialSTAGB300Processor&) = delete;

	const STAConfiguration<float>& config_;
	STAAcquisition<float>& acquisition_;
	std::vector<float> rxApod_;
	std::vector<float> txXY_, rxXY_, xyz_, value_, factor_;
	std::vector<unsigned int> txElems_;
	usgb_sta_params params_;
	usgb_ctx* ctx_ = nullptr;
};

class Vectorial3DSTAGB300Processor : public ArrayProcessor<XYZValueFactor<float>> {
public:
	Vectorial3DSTAGB300Processor(const SA3DConfiguration<float>& config, STAAcquisition<float>& acquisition,
			unsigned int upsamplingFactor, AnalyticSignalCoherenceFactorProcessor<float>& coherenceFactor,
			float peakOffset, const std::vector<float>& rxApod, uint32_t storage = USGB_STORE_F32)
		: config_(config), acquisition_(acquisition), rxApod_(rxApod), params_()
	{
		if (rxApod_.size() != config_.activeRxElem.size()) {
			THROW_EXCEPTION(InvalidValueException, "Wrong rx apodization size: " << rxApod_.size()
					<< " (should be " << config_.activeRxElem.size() << ").");
		}
		params_.num_tx = static_cast<uint32_t>(config_.activeTxElem.size());
		params_.num_rx = static_cast<uint32_t>(config_.activeRxElem.size());
		params_.upsampling = upsamplingFactor;
		params_.signal_path = USGB_PATH_ANALYTIC;
		params_.sampling_frequency = config_.samplingFrequency;
		params_.propagation_speed = config_.propagationSpeed;
		params_.center_frequency = config_.centerFrequency;
		params_.peak_offset = peakOffset;
		params_.dead_zone_m = config_.deadZoneM;
		params_.coherence = usgb_detail::analytic_cf(coherenceFactor, params_.pcf_gamma);
		params_.storage = storage;
		setBase(0);
	}
	virtual ~Vectorial3DSTAGB300Processor() { usgb_destroy(ctx_); }

	virtual void prepare(unsigned int baseElement)
	{
		if (baseElement != base_) {  // element positions change with the base element
			usgb_destroy(ctx_);
			ctx_ = nullptr;
			setBase(baseElement);
		}
		acquisition_.prepare(baseElement);
	}
	virtual void process(Matrix<XYZValueFactor<float>>& gridData)
	{
		usgb_detail::run_frame(ctx_, params_, txXY_, rxXY_, rxApod_, acquisition_, config_.activeTxElem, gridData,
				xyz_, value_, factor_);
	}
private:
	void setBase(unsigned int base)
	{
		base_ = base;
		txXY_.clear();
		rxXY_.clear();
		for (unsigned e : config_.activeTxElem) {
			txXY_.push_back(config_.txElemPos[base + e].x);
			txXY_.push_back(config_.txElemPos[base + e].y);
		}
		for (unsigned e : config_.activeRxElem) {
			rxXY_.push_back(config_.rxElemPos[base + e].x);
			rxXY_.push_back(config_.rxElemPos[base + e].y);
		}
	}

	const SA3DConfiguration<float>& config_;
	STAAcquisition<float>& acquisition_;
	std::vector<float> rxApod_;
	std::vector<float> txXY_, rxXY_, xyz_, value_, factor_;
	usgb_sta_params params_;
	usgb_ctx* ctx_ = nullptr;
	unsigned int base_ = 0;
};

class DefaultSTAGB300Processor : public ArrayProcessor<XYZValueFactor<float>> {
public:
	DefaultSTAGB300Processor(const STAConfiguration<float>& config, STAAcquisition<float>& acquisition,
			CoherenceFactorProcessor<float>& coherenceFactor, float peakOffset, float scfP = 1.0f)
		: config_(config), acquisition_(acquisition), params_()
	{
		std::vector<float> x;
		ArrayGeometry::getElementXCentered2D(config_.numElements, config_.pitch, x);
		for (unsigned e = 0; e < config_.numElements; ++e) {
			rxXY_.push_back(x[e]);
			rxXY_.push_back(0.0f);
		}
		for (unsigned e = config_.firstTxElem; e <= config_.lastTxElem; ++e) {
			txXY_.push_back(x[e]);
			txXY_.push_back(0.0f);
			txElems_.push_back(e);
		}
		params_.num_tx = static_cast<uint32_t>(txElems_.size());
		params_.num_rx = config_.numElements;
		params_.upsampling = 4;
		params_.signal_path = USGB_PATH_REAL;
		params_.sampling_frequency = config_.samplingFrequency;
		params_.propagation_speed = config_.propagationSpeed;
		params_.center_frequency = config_.centerFrequency;
		params_.peak_offset = peakOffset;
		params_.dead_zone_m = config_.deadZoneM;
		// CoherenceFactorProcessor does not expose its exponent; the caller
		// passes sign_coherence_factor_p (the same ParameterMap key).
		params_.coherence = coherenceFactor.enabled() ? USGB_CF_SCF : USGB_CF_NONE;
		params_.scf_p = scfP;
	}
	virtual ~DefaultSTAGB300Processor() { usgb_destroy(ctx_); }

	virtual void prepare(unsigned int baseElement) { acquisition_.prepare(baseElement); }
	virtual void process(Matrix<XYZValueFactor<float>>& gridData)
	{
		const std::vector<float> noApod;
		usgb_detail::run_frame(ctx_, params_, txXY_, rxXY_, noApod, acquisition_, txElems_, gridData, xyz_,
				value_, factor_);
	}
private:
	const STAConfiguration<float>& config_;
	STAAcquisition<float>& acquisition_;
	std::vector<float> txXY_, rxXY_, xyz_, value_, factor_;
	std::vector<unsigned int> txElems_;
	usgb_sta_params params_;
	usgb_ctx* ctx_ = nullptr;
};

}  // namespace Lab

#endif  // USGB_STA_PROCESSOR_HPP
