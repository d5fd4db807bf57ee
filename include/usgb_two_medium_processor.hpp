// Drop-in two-medium imaging processor for the reference tree (us_lab4a),
// built on the usgb_two_medium_* C ABI of usgb.h. Header-only; include it
// from a translation unit that sees the reference's headers
// (TwoMediumSTAConfiguration.h, Tensor3.h, Matrix.h, XZ.h, CoherenceFactor.h,
// Exception.h) and link libusgb.so.
//
//   VectorialCombinedTwoMediumImagingGB300Processor  same constructor, StepConfiguration
//       and process() as VectorialCombinedTwoMediumImagingProcessor<float>
//       (src/user/processor/VectorialCombinedTwoMediumImagingProcessor.h:59-90),
//       plus the storage type of the prepared signals
//
// Library status codes are rethrown as the reference's exception types.
#ifndef USGB_TWO_MEDIUM_PROCESSOR_HPP
#define USGB_TWO_MEDIUM_PROCESSOR_HPP

#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include "usgb.h"

namespace Lab {

class VectorialCombinedTwoMediumImagingGB300Processor {
public:
	struct StepConfiguration {
		unsigned int baseElemIdx;
		unsigned int baseElem;
		unsigned int firstTxElem;
		unsigned int lastTxElem;
	};

	VectorialCombinedTwoMediumImagingGB300Processor(const TwoMediumSTAConfiguration<float>& config,
			std::vector<Tensor3<float>>& acqDataList, unsigned int upsamplingFactor,
			AnalyticSignalCoherenceFactorProcessor<float>& coherenceFactor, float maxFermatBlockSize, float peakOffset,
			unsigned int signalStartOffset, uint32_t storage = USGB_STORE_F32)
		: acqDataList_(acqDataList)
	{
		if (acqDataList_.empty()) THROW_EXCEPTION(InvalidParameterException, "Empty acquisition list.");
		usgb_two_medium_params p{};
		p.num_elements = config.numElements;
		p.num_elements_mux = config.numElementsMux;
		p.pitch = config.pitch;
		p.center_frequency = config.centerFrequency;
		p.propagation_speed_1 = config.propagationSpeed1;
		p.propagation_speed_2 = config.propagationSpeed2;
		p.sampling_frequency = config.samplingFrequency;
		p.num_samples = static_cast<uint32_t>(acqDataList_[0].n3());
		p.upsampling = upsamplingFactor;
		p.max_fermat_block_size = maxFermatBlockSize;
		p.peak_offset = peakOffset;
		p.signal_start_offset = signalStartOffset;
		p.num_acquisitions = static_cast<uint32_t>(acqDataList_.size());
		p.num_tx = static_cast<uint32_t>(acqDataList_[0].n1());
		p.coherence = USGB_CF_NONE;
		if (coherenceFactor.enabled()) {
			std::vector<float> constants;
			coherenceFactor.implementation().getConstants(constants);  // {gamma, sigma0, gamma / sigma0}
			p.coherence = USGB_CF_PCF;
			p.pcf_gamma = constants.at(0);
		}
		p.storage = storage;
		check(usgb_two_medium_create(&p, &h_), nullptr);
	}
	~VectorialCombinedTwoMediumImagingGB300Processor() { usgb_two_medium_destroy(h_); }

	void process(const std::vector<StepConfiguration>& stepConfigList, const std::vector<XZ<float>>& interfacePointList,
			const std::vector<float>& rxApod, const Matrix<XZ<float>>& gridXZ, Matrix<std::complex<float>>& gridValue)
	{
		if (stepConfigList.empty()) THROW_EXCEPTION(InvalidParameterException, "The list of step configurations is empty.");
		if (gridXZ.n1() != gridValue.n1() || gridXZ.n2() != gridValue.n2()) {
			THROW_EXCEPTION(InvalidParameterException, "gridXZ and gridValue have different sizes.");
		}
		const Tensor3<float>& first = acqDataList_[0];
		const std::size_t acqSize = first.n1() * first.n2() * first.n3();
		rf_.resize(acqSize * acqDataList_.size());
		for (std::size_t a = 0; a < acqDataList_.size(); ++a) {
			const Tensor3<float>& t = acqDataList_[a];
			if (t.n1() != first.n1() || t.n2() != first.n2() || t.n3() != first.n3()) {
				THROW_EXCEPTION(InvalidParameterException, "The acquisitions differ in size.");
			}
			std::memcpy(&rf_[a * acqSize], &t(0, 0, 0), acqSize * sizeof(float));
		}
		steps_.resize(stepConfigList.size());
		for (std::size_t i = 0; i < stepConfigList.size(); ++i) {
			const StepConfiguration& s = stepConfigList[i];
			steps_[i] = {s.baseElemIdx, s.baseElem, s.firstTxElem, s.lastTxElem};
		}
		iface_.resize(2 * interfacePointList.size());
		for (std::size_t i = 0; i < interfacePointList.size(); ++i) {
			iface_[2 * i] = interfacePointList[i].x;
			iface_[2 * i + 1] = interfacePointList[i].z;
		}
		const std::size_t n = gridXZ.size();
		grid_.resize(2 * n);
		for (std::size_t i = 0; i < n; ++i) {
			grid_[2 * i] = (gridXZ.data() + i)->x;
			grid_[2 * i + 1] = (gridXZ.data() + i)->z;
		}
		out_.resize(2 * n);
		check(usgb_two_medium_process(h_, rf_.data(), steps_.data(), static_cast<uint32_t>(steps_.size()), iface_.data(),
				static_cast<uint32_t>(interfacePointList.size()), rxApod.data(), grid_.data(),
				static_cast<uint32_t>(gridXZ.n1()), static_cast<uint32_t>(gridXZ.n2()), out_.data()), h_);
		for (std::size_t i = 0; i < n; ++i) *(gridValue.data() + i) = std::complex<float>(out_[2 * i], out_[2 * i + 1]);
	}
private:
	VectorialCombinedTwoMediumImagingGB300Processor(const VectorialCombinedTwoMediumImagingGB300Processor&) = delete;
	VectorialCombinedTwoMediumImagingGB300Processor& operator=(const VectorialCombinedTwoMediumImagingGB300Processor&) = delete;

	static void check(int rc, const usgb_two_medium* h)
	{
		if (rc == USGB_OK) return;
		const std::string msg = usgb_two_medium_last_error(h);
		switch (rc) {
		case USGB_ERR_INVALID_PARAMETER: THROW_EXCEPTION(InvalidParameterException, msg);
		case USGB_ERR_INVALID_VALUE: THROW_EXCEPTION(InvalidValueException, msg);
		case USGB_ERR_INVALID_STATE: THROW_EXCEPTION(InvalidStateException, msg);
		default: THROW_EXCEPTION(Exception, "[usgb " << rc << "] " << msg);
		}
	}

	std::vector<Tensor3<float>>& acqDataList_;
	std::vector<float> rf_, iface_, grid_, out_;
	std::vector<usgb_two_medium_step> steps_;
	usgb_two_medium* h_ = nullptr;
};

}  // namespace Lab

#endif  // USGB_TWO_MEDIUM_PROCESSOR_HPP
