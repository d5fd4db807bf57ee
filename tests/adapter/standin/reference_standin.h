// Test infrastructure: stand-ins for the few types of the reference tree
// (us_lab4a, namespace Lab) that the drop-in processor headers use, so that
// include/usgb_sta_processor.hpp compiles and runs where the reference
// sources are absent (the GPU host). Names, members and meaning follow the
// reference's interface; the implementations are minimal and our own:
//   Exception, InvalidParameterException, InvalidValueException,
//   InvalidStateException, THROW_EXCEPTION      src/util/Exception.h
//   Matrix<T> (element (i, j) at i * n2 + j)    src/util/Matrix.h
//   XY<T>, XYZValueFactor<T>                    src/util/XY.h, src/util/XYZValueFactor.h
//   Util::resetValueFactor                      src/util/Util.h:990-999
//   ArrayGeometry::getElementXCentered2D        src/util/ArrayGeometry.h:37-50
//   ArrayProcessor<TPoint>                      src/user/processor/ArrayProcessor.h:28-40
//   STAAcquisition<TFloat>                      src/user/acquisition/STAAcquisition.h:28-42
//   STAConfiguration<TFloat>                    src/user/configuration/STAConfiguration.h:29-51
//   SA3DConfiguration<TFloat>                   src/user/configuration/SA3DConfiguration.h
//   AnalyticSignalCoherenceFactor(Processor), CoherenceFactorProcessor
//                                               src/util/CoherenceFactor.h
// The coherence-factor processors are built here from their constants (the
// reference builds them from a ParameterMap).
#ifndef USGB_REFERENCE_STANDIN_H
#define USGB_REFERENCE_STANDIN_H

#include <cstddef>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace Lab {

class Exception : public std::runtime_error {
public:
	explicit Exception(const std::string& msg) : std::runtime_error(msg) {}
};
class InvalidParameterException : public Exception { public: using Exception::Exception; };
class InvalidValueException : public Exception { public: using Exception::Exception; };
class InvalidStateException : public Exception { public: using Exception::Exception; };

#define THROW_EXCEPTION(E, M)                 \
	do {                                      \
		std::ostringstream usgbStandinMsg_;   \
		usgbStandinMsg_ << M;                 \
		throw E(usgbStandinMsg_.str());       \
	} while (0)

template<typename T>
class Matrix {
public:
	using Iterator = typename std::vector<T>::iterator;
	Matrix() = default;
	Matrix(std::size_t n1, std::size_t n2) { resize(n1, n2); }
	void resize(std::size_t n1, std::size_t n2)
	{
		n1_ = n1;
		n2_ = n2;
		v_.resize(n1 * n2);
	}
	std::size_t n1() const { return n1_; }
	std::size_t n2() const { return n2_; }
	std::size_t size() const { return v_.size(); }
	T* data() { return v_.data(); }
	const T* data() const { return v_.data(); }
	Iterator begin() { return v_.begin(); }
	Iterator end() { return v_.end(); }
	T& operator()(std::size_t i, std::size_t j) { return v_[i * n2_ + j]; }
	const T& operator()(std::size_t i, std::size_t j) const { return v_[i * n2_ + j]; }
private:
	std::size_t n1_ = 0, n2_ = 0;
	std::vector<T> v_;
};

template<typename T> struct XY { T x; T y; };

template<typename T>
struct XYZValueFactor {
	T x, y, z, value, factor;
	XYZValueFactor() : x(), y(), z(), value(), factor(1) {}
};

namespace Util {
template<typename Iterator>
void resetValueFactor(Iterator iter, Iterator iterEnd)
{
	for (; iter != iterEnd; ++iter) {
		iter->value = 0;
		iter->factor = 1;
	}
}
}  // namespace Util

namespace ArrayGeometry {
template<typename TFloat>
void getElementXCentered2D(unsigned int numElements, TFloat pitch, std::vector<TFloat>& x)
{
	if (numElements == 0) THROW_EXCEPTION(InvalidParameterException, "The number of elements is zero.");
	x.resize(numElements);
	const TFloat xCenter = ((numElements - 1) * pitch) / 2;
	for (unsigned int e = 0; e < numElements; ++e) x[e] = e * pitch - xCenter;
}
}  // namespace ArrayGeometry

template<typename TPoint>
class ArrayProcessor {
public:
	ArrayProcessor() = default;
	virtual ~ArrayProcessor() = default;
	virtual void prepare(unsigned int) {}
	virtual void process(Matrix<TPoint>& gridData) = 0;
	ArrayProcessor(const ArrayProcessor&) = delete;
	ArrayProcessor& operator=(const ArrayProcessor&) = delete;
};

template<typename TFloat>
class STAAcquisition {
public:
	typedef Matrix<TFloat> AcquisitionDataType;
	STAAcquisition() = default;
	virtual ~STAAcquisition() = default;
	virtual void prepare(unsigned int) {}
	virtual void execute(unsigned int txElement, AcquisitionDataType& acqData) = 0;
	STAAcquisition(const STAAcquisition&) = delete;
	STAAcquisition& operator=(const STAAcquisition&) = delete;
};

template<typename TFloat>
struct STAConfiguration {
	unsigned int numElements = 0, numElementsMux = 0, firstTxElem = 0, lastTxElem = 0, numPulses = 1;
	TFloat pitch = 0, centerFrequency = 0, maxFrequency = 0, acquisitionTime = 0, minGain = 0, maxGain = 0;
	TFloat propagationSpeed = 0, acquisitionDelay = 0, samplingFrequency = 0, deadZoneM = 0, valueScale = 1;
};

template<typename TFloat>
struct SA3DConfiguration {
	unsigned int numElements = 0, numElementsMux = 0, numPulses = 1;
	TFloat centerFrequency = 0, maxFrequency = 0, acquisitionTime = 0, minGain = 0, maxGain = 0;
	TFloat propagationSpeed = 0, acquisitionDelay = 0, samplingFrequency = 0, deadZoneM = 0, valueScale = 1;
	std::vector<unsigned int> activeTxElem, activeRxElem;
	std::vector<XY<TFloat>> txElemPos, rxElemPos;
};

// getConstants of the phase coherence factor: {gamma, sigma0, gamma / sigma0}
// (src/util/CoherenceFactor.h:288-295).
template<typename TFloat>
class AnalyticSignalCoherenceFactor {
public:
	explicit AnalyticSignalCoherenceFactor(TFloat gamma) : gamma_(gamma) {}
	void getConstants(std::vector<TFloat>& list) const
	{
		const TFloat sigma0 = 3.14159265358979323846 / 1.7320508075688772;
		list = {gamma_, sigma0, gamma_ / sigma0};
	}
private:
	TFloat gamma_;
};

template<typename TFloat>
class AnalyticSignalCoherenceFactorProcessor {
public:
	AnalyticSignalCoherenceFactorProcessor() = default;   // no coherence factor
	explicit AnalyticSignalCoherenceFactorProcessor(TFloat pcfGamma)
		: cf_(new AnalyticSignalCoherenceFactor<TFloat>(pcfGamma)) {}
	bool enabled() const { return cf_ != nullptr; }
	const AnalyticSignalCoherenceFactor<TFloat>& implementation() const { return *cf_; }
private:
	std::unique_ptr<AnalyticSignalCoherenceFactor<TFloat>> cf_;
};

template<typename TFloat>
class CoherenceFactorProcessor {
public:
	CoherenceFactorProcessor() = default;   // no coherence factor
	explicit CoherenceFactorProcessor(bool scf) : enabled_(scf) {}
	bool enabled() const { return enabled_; }
private:
	bool enabled_ = false;
};

}  // namespace Lab

#endif  // USGB_REFERENCE_STANDIN_H
