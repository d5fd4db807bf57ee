// Drop-in single-term 3D processors for the reference tree (us_lab4a), built
// on the usgb_single_* C ABI of usgb.h. Header-only; include it from a
// translation unit that sees the reference's headers (ArrayProcessor.h,
// SA3DConfiguration.h, TnRnConfiguration.h, STAAcquisition.h,
// TnRnAcquisition.h, CoherenceFactor.h, Exception.h, Util.h) and link
// libusgb.so.
//
//   Vectorial3DT1R1SAFTGB300Processor   same constructor as Vectorial3DT1R1SAFTProcessor<float>
//                                       (src/user/processor/Vectorial3DT1R1SAFTProcessor.h:54-59)
//   Vectorial3DTnRnGB300Processor       same constructor, setTxDelays and prepare as
//                                       Vectorial3DTnRnProcessor<float>
//                                       (src/user/processor/Vectorial3DTnRnProcessor.h:54-66)
//   SynthYVectorial3DTnRnGB300Processor same interface as SynthYVectorial3DTnRnProcessor<float>
//                                       (src/user/processor/SynthYVectorial3DTnRnProcessor.h:54-68),
//                                       plus the number of acquisitions kept on the device
//
// As in the reference, the signal length comes from the first acquisition;
// library status codes are rethrown as the reference's exception types.
#ifndef USGB_SINGLE_PROCESSOR_HPP
#define USGB_SINGLE_PROCESSOR_HPP

#include <cstring>
#include <string>
#include <vector>

#include "usgb.h"

namespace Lab {

namespace usgb_single_detail {

inline void check(int rc, const usgb_single* h)
{
	if (rc == USGB_OK) return;
	const std::string msg = usgb_single_last_error(h);
	switch (rc) {
	case USGB_ERR_INVALID_PARAMETER: THROW_EXCEPTION(InvalidParameterException, msg);
	case USGB_ERR_INVALID_VALUE: THROW_EXCEPTION(InvalidValueException, msg);
	case USGB_ERR_INVALID_STATE: THROW_EXCEPTION(InvalidStateException, msg);
	default: THROW_EXCEPTION(Exception, "[usgb " << rc << "] " << msg);
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

// Grid coordinates to the library, value / factor back into gridData.
class GridIO {
public:
	void set(usgb_single* h, const Matrix<XYZValueFactor<float>>& gridData)
	{
		const std::size_t n = gridData.size();
		std::vector<float> xyz(3 * n);
		for (std::size_t p = 0; p < n; ++p) {
			const XYZValueFactor<float>& point = *(gridData.data() + p);
			xyz[3 * p] = point.x;
			xyz[3 * p + 1] = point.y;
			xyz[3 * p + 2] = point.z;
		}
		if (xyz != xyz_ || h != h_) {
			check(usgb_single_set_grid(h, xyz.data(), static_cast<uint32_t>(gridData.n1()),
					static_cast<uint32_t>(gridData.n2())), h);
			xyz_.swap(xyz);
			h_ = h;
		}
		value_.resize(n);
		factor_.resize(n);
	}
	void store(Matrix<XYZValueFactor<float>>& gridData) const
	{
		for (std::size_t p = 0; p < gridData.size(); ++p) {
			XYZValueFactor<float>& point = *(gridData.data() + p);
			point.value = value_[p];
			point.factor = factor_[p];
		}
	}
	float* value() { return value_.data(); }
	float* factor() { return factor_.data(); }
private:
	std::vector<float> xyz_, value_, factor_;
	const usgb_single* h_ = nullptr;
};

}  // namespace usgb_single_detail

class Vectorial3DT1R1SAFTGB300Processor : public ArrayProcessor<XYZValueFactor<float>> {
public:
	Vectorial3DT1R1SAFTGB300Processor(const SA3DConfiguration<float>& config, STAAcquisition<float>& acquisition,
			unsigned int upsamplingFactor, AnalyticSignalCoherenceFactorProcessor<float>& coherenceFactor,
			float peakOffset, uint32_t storage = USGB_STORE_F32)
		: config_(config), acquisition_(acquisition), params_()
	{
		if (config_.activeTxElem.size() != config_.activeRxElem.size()) {
			THROW_EXCEPTION(InvalidParameterException, "The number of active tx and rx elements differ.");
		}
		params_.mode = USGB_SINGLE_T1R1_SAFT;
		params_.num_signals = static_cast<uint32_t>(config_.activeTxElem.size());
		params_.upsampling = upsamplingFactor;
		params_.sampling_frequency = config_.samplingFrequency;
		params_.propagation_speed = config_.propagationSpeed;
		params_.center_frequency = config_.centerFrequency;
		params_.peak_offset = peakOffset;
		params_.dead_zone_m = config_.deadZoneM;
		params_.coherence = usgb_single_detail::analytic_cf(coherenceFactor, params_.pcf_gamma);
		params_.storage = storage;
	}
	virtual ~Vectorial3DT1R1SAFTGB300Processor() { usgb_single_destroy(h_); }

	virtual void prepare(unsigned int baseElement)
	{
		if (baseElement != base_) {  // element positions change with the base element
			usgb_single_destroy(h_);
			h_ = nullptr;
			base_ = baseElement;
		}
		acquisition_.prepare(baseElement);
	}
	virtual void process(Matrix<XYZValueFactor<float>>& gridData)
	{
		Util::resetValueFactor(gridData.begin(), gridData.end());
		const std::size_t n = config_.activeTxElem.size();
		for (std::size_t i = 0; i < n; ++i) {
			acquisition_.execute(config_.activeTxElem[i], acqData_);
			const std::size_t ns = acqData_.n2();
			if (!h_) {
				txXY_.clear();
				rxXY_.clear();
				for (std::size_t k = 0; k < n; ++k) {
					const auto& t = config_.txElemPos[base_ + config_.activeTxElem[k]];
					const auto& r = config_.rxElemPos[base_ + config_.activeRxElem[k]];
					txXY_.insert(txXY_.end(), {t.x, t.y});
					rxXY_.insert(rxXY_.end(), {r.x, r.y});
				}
				params_.num_samples = static_cast<uint32_t>(ns);
				params_.tx_xy = txXY_.data();
				params_.rx_xy = rxXY_.data();
				usgb_single_detail::check(usgb_single_create(&params_, &h_), nullptr);
				rf_.assign(n * ns, 0.0f);
			} else if (ns != params_.num_samples) {
				THROW_EXCEPTION(InvalidValueException, "Data size mismatch.");
			}
			std::memcpy(&rf_[i * ns], &acqData_(0, 0), ns * sizeof(float));  // the first row, as the reference
		}
		io_.set(h_, gridData);
		usgb_single_detail::check(usgb_single_process(h_, rf_.data(), io_.value(), io_.factor()), h_);
		io_.store(gridData);
	}
private:
	Vectorial3DT1R1SAFTGB300Processor(const Vectorial3DT1R1SAFTGB300Processor&) = delete;
	Vectorial3DT1R1SAFTGB300Processor& operator=(const Vectorial3DT1R1SAFTGB300Processor&) = delete;

	const SA3DConfiguration<float>& config_;
	STAAcquisition<float>& acquisition_;
	typename STAAcquisition<float>::AcquisitionDataType acqData_;
	usgb_single_params params_;
	std::vector<float> txXY_, rxXY_, rf_;
	usgb_single_detail::GridIO io_;
	usgb_single* h_ = nullptr;
	unsigned int base_ = 0;
};

namespace usgb_single_detail {

// Shared part of the TnRn processors: parameters, tx focus, context.
class TnRnBase {
protected:
	TnRnBase(const TnRnConfiguration<float>& config, TnRnAcquisition<float>& acquisition, unsigned int upsamplingFactor,
			AnalyticSignalCoherenceFactorProcessor<float>& coherenceFactor, float peakOffset,
			const std::vector<float>& rxApod, uint32_t mode, uint32_t storage, uint32_t maxAcquisitions)
		: config_(config), acquisition_(acquisition), rxApod_(rxApod), params_()
	{
		if (rxApod_.size() != config_.numElements) {
			THROW_EXCEPTION(InvalidValueException, "Wrong rx apodization size: " << rxApod_.size()
					<< " (should be " << config_.numElements << ").");
		}
		params_.mode = mode;
		params_.num_signals = config_.numElements;
		params_.upsampling = upsamplingFactor;
		params_.sampling_frequency = config_.samplingFrequency;
		params_.propagation_speed = config_.propagationSpeed;
		params_.center_frequency = config_.centerFrequency;
		params_.peak_offset = peakOffset;
		params_.dead_zone_m = config_.deadZoneM;
		params_.coherence = analytic_cf(coherenceFactor, params_.pcf_gamma);
		params_.storage = storage;
		params_.max_acquisitions = maxAcquisitions;
	}
	~TnRnBase() { usgb_single_destroy(h_); }

	void setTxDelaysImpl(float focusX, float focusY, float focusZ, const std::vector<float>& txDelays)
	{
		focusX_ = focusX;
		focusY_ = focusY;
		focusZ_ = focusZ;
		txDelays_ = txDelays;
		if (h_ && !txDelays_.empty()) {
			check(usgb_single_set_tx_delays(h_, focusX_, focusY_, focusZ_, txDelays_.data(),
					static_cast<uint32_t>(txDelays_.size())), h_);
		}
	}
	void prepareImpl(unsigned int baseElement)
	{
		if (baseElement + config_.numElements > config_.numElementsMux) {
			THROW_EXCEPTION(InvalidParameterException, "Invalid base element: " << baseElement << '.');
		}
		if (txDelays_.empty()) THROW_EXCEPTION(InvalidStateException, "Empty tx delay list.");
		if (baseElement != base_) {
			usgb_single_destroy(h_);
			h_ = nullptr;
			base_ = baseElement;
		}
		acquisition_.prepare(baseElement, txDelays_);
	}
	// Acquires one RF block; creates the context on the first one.
	void acquire()
	{
		acquisition_.execute(acqData_);
		if (acqData_.n1() != config_.numElements) THROW_EXCEPTION(InvalidValueException, "Data size mismatch.");
		if (!h_) {
			txXY_ = {config_.txElemPos[base_].x, config_.txElemPos[base_].y};
			rxXY_.clear();
			for (unsigned e = 0; e < config_.numElements; ++e) {
				rxXY_.insert(rxXY_.end(), {config_.rxElemPos[base_ + e].x, config_.rxElemPos[base_ + e].y});
			}
			params_.num_samples = static_cast<uint32_t>(acqData_.n2());
			params_.tx_xy = txXY_.data();
			params_.rx_xy = rxXY_.data();
			params_.rx_apod = rxApod_.data();
			check(usgb_single_create(&params_, &h_), nullptr);
			check(usgb_single_set_tx_delays(h_, focusX_, focusY_, focusZ_, txDelays_.data(),
					static_cast<uint32_t>(txDelays_.size())), h_);
		} else if (acqData_.n2() != params_.num_samples) {
			THROW_EXCEPTION(InvalidValueException, "Data size mismatch.");
		}
	}

	const TnRnConfiguration<float>& config_;
	TnRnAcquisition<float>& acquisition_;
	typename TnRnAcquisition<float>::AcquisitionDataType acqData_;
	std::vector<float> rxApod_, txXY_, rxXY_, txDelays_;
	float focusX_ = 0, focusY_ = 0, focusZ_ = 0;
	usgb_single_params params_;
	GridIO io_;
	usgb_single* h_ = nullptr;
	unsigned int base_ = 0;
};

}  // namespace usgb_single_detail

class Vectorial3DTnRnGB300Processor : public ArrayProcessor<XYZValueFactor<float>>, private usgb_single_detail::TnRnBase {
public:
	Vectorial3DTnRnGB300Processor(const TnRnConfiguration<float>& config, TnRnAcquisition<float>& acquisition,
			unsigned int upsamplingFactor, AnalyticSignalCoherenceFactorProcessor<float>& coherenceFactor,
			float peakOffset, const std::vector<float>& rxApod, uint32_t storage = USGB_STORE_F32)
		: TnRnBase(config, acquisition, upsamplingFactor, coherenceFactor, peakOffset, rxApod, USGB_SINGLE_TNRN,
				storage, 0) {}
	virtual ~Vectorial3DTnRnGB300Processor() = default;

	void setTxDelays(float focusX, float focusY, float focusZ, const std::vector<float>& txDelays)
	{
		setTxDelaysImpl(focusX, focusY, focusZ, txDelays);
	}
	virtual void prepare(unsigned int baseElement) { prepareImpl(baseElement); }
	virtual void process(Matrix<XYZValueFactor<float>>& gridData)
	{
		Util::resetValueFactor(gridData.begin(), gridData.end());
		acquire();
		io_.set(h_, gridData);
		usgb_single_detail::check(usgb_single_process(h_, &acqData_(0, 0), io_.value(), io_.factor()), h_);
		io_.store(gridData);
	}
};

class SynthYVectorial3DTnRnGB300Processor : private usgb_single_detail::TnRnBase {
public:
	SynthYVectorial3DTnRnGB300Processor(const TnRnConfiguration<float>& config, TnRnAcquisition<float>& acquisition,
			unsigned int upsamplingFactor, AnalyticSignalCoherenceFactorProcessor<float>& coherenceFactor,
			float peakOffset, const std::vector<float>& rxApod, uint32_t maxAcquisitions = 64,
			uint32_t storage = USGB_STORE_F32)
		: TnRnBase(config, acquisition, upsamplingFactor, coherenceFactor, peakOffset, rxApod,
				USGB_SINGLE_SYNTH_Y_TNRN, storage, maxAcquisitions) {}

	void setTxDelays(float focusX, float focusY, float focusZ, const std::vector<float>& txDelays)
	{
		setTxDelaysImpl(focusX, focusY, focusZ, txDelays);
	}
	void prepare(unsigned int baseElement) { prepareImpl(baseElement); }
	void getAcqData(float y)
	{
		acquire();
		usgb_single_detail::check(usgb_single_add_acquisition(h_, &acqData_(0, 0), y), h_);
		y_.push_back(y);
	}
	void process(unsigned int firstAcq, unsigned int lastAcq, Matrix<XYZValueFactor<float>>& gridData)
	{
		if (txDelays_.empty()) THROW_EXCEPTION(InvalidStateException, "Empty tx delay list.");
		if (!h_) THROW_EXCEPTION(InvalidStateException, "No acquisition data.");
		Util::resetValueFactor(gridData.begin(), gridData.end());
		io_.set(h_, gridData);
		usgb_single_detail::check(usgb_single_process_window(h_, firstAcq, lastAcq, io_.value(), io_.factor()), h_);
		io_.store(gridData);
		const float centerY = y_[(firstAcq + lastAcq) / 2U];
		for (auto it = gridData.begin(); it != gridData.end(); ++it) it->y = centerY;
	}
private:
	std::vector<float> y_;
};

}  // namespace Lab

#endif  // USGB_SINGLE_PROCESSOR_HPP
