// Driver that runs the reference's own processors, compiled from their
// unchanged sources (src/user/processor/{VectorialSTAProcessor,
// Vectorial3DSTAProcessor,DefaultSTAProcessor,Vectorial3DT1R1SAFTProcessor,
// Vectorial3DTnRnProcessor,SynthYVectorial3DTnRnProcessor,
// VectorialCombinedTwoMediumImagingProcessor}.h), on in-memory RF.
// TEST INFRASTRUCTURE ONLY: it produces golden outputs for the parity tests
// and validates the oracle restatement; nothing in the product uses it.
//
// The processors are constructed exactly as STAMethod / STA3DMethod construct
// them (src/user/method/STAMethod.cpp:191-229, STA3DMethod.cpp:146-163),
// with coherence-factor objects built from ParameterMap files the same way
// the reference's project files configure them.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <unistd.h>

#include "DefaultSTAProcessor.h"
#include "SynthYVectorial3DTnRnProcessor.h"
#include "TnRnAcquisition.h"
#include "TnRnConfiguration.h"
#include "Vectorial3DSTAProcessor.h"
#include "Vectorial3DT1R1SAFTProcessor.h"
#include "Vectorial3DTnRnProcessor.h"
#include "VectorialCombinedTwoMediumImagingProcessor.h"
#include "VectorialSTAProcessor.h"
#include "WindowFunction.h"
#include "XYZValueFactor.h"

using namespace Lab;

namespace {

thread_local std::string g_err;

// STAAcquisition over a caller-owned (numTx, numRx, numSamples) RF block.
template<typename T>
class MemoryAcquisition : public STAAcquisition<T> {
public:
	MemoryAcquisition(const T* rf, unsigned firstTx, unsigned numRx, unsigned ns)
		: rf_(rf), firstTx_(firstTx), numRx_(numRx), ns_(ns) {}
	void execute(unsigned int txElement, typename STAAcquisition<T>::AcquisitionDataType& acqData) override
	{
		acqData.resize(numRx_, ns_);
		const T* src = rf_ + static_cast<std::size_t>(txElement - firstTx_) * numRx_ * ns_;
		for (unsigned r = 0; r < numRx_; ++r) {
			for (unsigned s = 0; s < ns_; ++s) acqData(r, s) = src[static_cast<std::size_t>(r) * ns_ + s];
		}
	}
private:
	const T* rf_;
	unsigned firstTx_, numRx_, ns_;
};

// STAAcquisition of a T1R1 SAFT scan: one A-scan per active element, row i of
// `rf` for element active[i].
template<typename T>
class SaftAcquisition : public STAAcquisition<T> {
public:
	SaftAcquisition(const T* rf, const std::vector<unsigned>& active, unsigned ns) : rf_(rf), active_(active), ns_(ns) {}
	void execute(unsigned int txElement, typename STAAcquisition<T>::AcquisitionDataType& acqData) override
	{
		unsigned row = 0;
		while (row < active_.size() && active_[row] != txElement) ++row;
		if (row == active_.size()) throw std::runtime_error("element not in the active list");
		acqData.resize(1, ns_);
		for (unsigned s = 0; s < ns_; ++s) acqData(0, s) = rf_[static_cast<std::size_t>(row) * ns_ + s];
	}
private:
	const T* rf_;
	std::vector<unsigned> active_;
	unsigned ns_;
};

// TnRnAcquisition over a caller-owned (numElements, numSamples) RF block.
template<typename T>
class MemoryTnRnAcquisition : public TnRnAcquisition<T> {
public:
	MemoryTnRnAcquisition(const T* rf, unsigned numElements, unsigned ns) : rf_(rf), numElements_(numElements), ns_(ns) {}
	void setData(const T* rf) { rf_ = rf; }
	void execute(typename TnRnAcquisition<T>::AcquisitionDataType& acqData) override
	{
		acqData.resize(numElements_, ns_);
		for (unsigned r = 0; r < numElements_; ++r) {
			for (unsigned s = 0; s < ns_; ++s) acqData(r, s) = rf_[static_cast<std::size_t>(r) * ns_ + s];
		}
	}
private:
	const T* rf_;
	unsigned numElements_, ns_;
};

// Temporary key=value file for ParameterMap.
struct TempParamFile {
	std::string path;
	explicit TempParamFile(const std::string& text)
	{
		char tmpl[] = "/tmp/usgb_ref_pm_XXXXXX";
		const int fd = mkstemp(tmpl);
		if (fd < 0) throw std::runtime_error("mkstemp failed");
		close(fd);
		path = tmpl;
		std::ofstream out(path);
		out << text;
	}
	~TempParamFile() { std::remove(path.c_str()); }
};

template<typename T>
struct RefDesc {
	// 2D linear array (STAConfiguration) ...
	unsigned num_elements, first_tx_elem, last_tx_elem;
	T pitch;
	// ... or 3D matrix array (SA3DConfiguration), used when is_3d != 0.
	int is_3d;
	unsigned tx_nx, tx_ny, rx_nx, rx_ny;
	T tx_pitch_x, tx_pitch_y, rx_pitch_x, rx_pitch_y;
	// Common acquisition parameters.
	unsigned num_samples, upsampling;
	T sampling_frequency, propagation_speed, center_frequency, peak_offset, dead_zone_m;
	const T* rx_apod;
	int cf;  // 0 none, 1 PCF (analytic path), 2 SCF (real path)
	T pcf_gamma, scf_p;
	int real_path;
};

template<typename T>
void fill_config(const RefDesc<T>& d, STAConfiguration<T>& c)
{
	c.numElementsMux = d.num_elements;
	c.numElements = d.num_elements;
	c.firstTxElem = d.first_tx_elem;
	c.lastTxElem = d.last_tx_elem;
	c.numPulses = 1;
	c.pitch = d.pitch;
	c.centerFrequency = d.center_frequency;
	c.maxFrequency = d.center_frequency * 2;
	c.acquisitionTime = 1e-4;
	c.minGain = 0;
	c.maxGain = 0;
	c.propagationSpeed = d.propagation_speed;
	c.acquisitionDelay = 0;
	c.samplingFrequency = d.sampling_frequency;
	c.deadZoneM = d.dead_zone_m;
	c.valueScale = 1;
}

template<typename T>
int run(const RefDesc<T>* dp, const T* rf, const T* gridXYZ, unsigned n1, unsigned n2, T* value, T* factor)
{
	try {
		const RefDesc<T>& d = *dp;
		Matrix<XYZValueFactor<T>> grid(n1, n2);
		for (unsigned i = 0; i < n1; ++i) {
			for (unsigned j = 0; j < n2; ++j) {
				const std::size_t p = static_cast<std::size_t>(i) * n2 + j;
				grid(i, j).x = gridXYZ[3 * p];
				grid(i, j).y = gridXYZ[3 * p + 1];
				grid(i, j).z = gridXYZ[3 * p + 2];
			}
		}
		if (d.real_path) {
			STAConfiguration<T> c;
			fill_config(d, c);
			const unsigned numRx = c.numElements;
			MemoryAcquisition<T> acq(rf, c.firstTxElem, numRx, d.num_samples);
			std::string text = "coherence_factor_method = none\n";
			if (d.cf == 2) {
				text = "coherence_factor_method = sign_coherence_factor\nsign_coherence_factor_p = " +
						std::to_string(static_cast<double>(d.scf_p)) + "\n";
			}
			TempParamFile f(text);
			ParameterMap pm(f.path);
			CoherenceFactorProcessor<T> cf(pm);
			DefaultSTAProcessor<T, XYZValueFactor<T>> proc(c, acq, cf, d.peak_offset);
			proc.prepare(0);
			proc.process(grid);
		} else {
			std::string text = "analytic_signal_coherence_factor_method = none\n";
			if (d.cf == 1) {
				char buf[64];
				std::snprintf(buf, sizeof buf, "%.17g", static_cast<double>(d.pcf_gamma));
				text = std::string("analytic_signal_coherence_factor_method = phase_coherence_factor\n"
						"phase_coherence_factor_gamma = ") + buf + "\n";
			}
			TempParamFile f(text);
			ParameterMap pm(f.path);
			AnalyticSignalCoherenceFactorProcessor<T> cf(pm);
			if (d.is_3d) {
				SA3DConfiguration<T> c;
				c.numElementsMux = 1024;
				c.numPulses = 1;
				c.centerFrequency = d.center_frequency;
				c.maxFrequency = d.center_frequency * 2;
				c.acquisitionTime = 1e-4;
				c.minGain = 0;
				c.maxGain = 0;
				c.propagationSpeed = d.propagation_speed;
				c.acquisitionDelay = 0;
				c.samplingFrequency = d.sampling_frequency;
				c.deadZoneM = d.dead_zone_m;
				c.valueScale = 1;
				ArrayUtil::calculateElementPositions(d.tx_pitch_x, d.tx_nx, T(0), d.tx_pitch_y, d.tx_ny, T(0), c.txElemPos);
				ArrayUtil::calculateElementPositions(d.rx_pitch_x, d.rx_nx, T(0), d.rx_pitch_y, d.rx_ny, T(0), c.rxElemPos);
				for (unsigned i = 0; i < c.txElemPos.size(); ++i) c.activeTxElem.push_back(i);
				for (unsigned i = 0; i < c.rxElemPos.size(); ++i) c.activeRxElem.push_back(i);
				const unsigned numRx = static_cast<unsigned>(c.rxElemPos.size());
				std::vector<T> apod(d.rx_apod, d.rx_apod + numRx);
				MemoryAcquisition<T> acq(rf, 0, numRx, d.num_samples);
				Vectorial3DSTAProcessor<T> proc(c, acq, d.upsampling, cf, d.peak_offset, apod);
				proc.prepare(0);
				proc.process(grid);
			} else {
				STAConfiguration<T> c;
				fill_config(d, c);
				const unsigned numRx = c.numElements;
				std::vector<T> apod(d.rx_apod, d.rx_apod + numRx);
				MemoryAcquisition<T> acq(rf, c.firstTxElem, numRx, d.num_samples);
				VectorialSTAProcessor<T, XYZValueFactor<T>> proc(c, acq, d.upsampling, cf, d.peak_offset, apod);
				proc.prepare(0);
				proc.process(grid);
			}
		}
		for (unsigned i = 0; i < n1; ++i) {
			for (unsigned j = 0; j < n2; ++j) {
				const std::size_t p = static_cast<std::size_t>(i) * n2 + j;
				value[p] = grid(i, j).value;
				factor[p] = grid(i, j).factor;
			}
		}
		return 0;
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

template<typename T>
struct RefSingleDesc {
	int mode;                  // 0 T1R1 SAFT, 1 TnRn, 2 synthetic-y TnRn
	unsigned nx, ny;           // matrix array (ArrayUtil::calculateElementPositions, no offset); tx = rx
	T pitch_x, pitch_y;
	unsigned num_active;       // T1R1: active elements (tx list = rx list)
	const unsigned* active;    // T1R1: the active element numbers
	unsigned base_element;     // TnRn: base element of the group
	unsigned num_elements;     // TnRn: group size
	unsigned num_samples, upsampling;
	T sampling_frequency, propagation_speed, center_frequency, peak_offset, dead_zone_m;
	const T* rx_apod;          // TnRn: num_elements weights
	T focus_x, focus_y, focus_z;
	unsigned num_acq;          // synthetic y: acquisitions in rf (num_acq x num_elements x num_samples)
	const T* acq_y;            // synthetic y: num_acq positions
	unsigned first_acq, last_acq;
	int cf;                    // 0 none, 1 PCF
	T pcf_gamma;
	T* tx_delays_out;          // TnRn: the group's focusing delays (s), num_elements; may be NULL
};

template<typename T>
void fill_common(const RefSingleDesc<T>& d, T& fc, T& maxF, T& acqTime, T& minGain, T& maxGain, T& c, T& acqDelay, T& fs, T& dz, T& vs)
{
	fc = d.center_frequency;
	maxF = d.center_frequency * 2;
	acqTime = 1e-4;
	minGain = 0;
	maxGain = 0;
	c = d.propagation_speed;
	acqDelay = 0;
	fs = d.sampling_frequency;
	dz = d.dead_zone_m;
	vs = 1;
}

template<typename T>
int run_single(const RefSingleDesc<T>* dp, const T* rf, const T* gridXYZ, unsigned n1, unsigned n2, T* value, T* factor)
{
	try {
		const RefSingleDesc<T>& d = *dp;
		Matrix<XYZValueFactor<T>> grid(n1, n2);
		for (unsigned i = 0; i < n1; ++i) {
			for (unsigned j = 0; j < n2; ++j) {
				const std::size_t p = static_cast<std::size_t>(i) * n2 + j;
				grid(i, j).x = gridXYZ[3 * p];
				grid(i, j).y = gridXYZ[3 * p + 1];
				grid(i, j).z = gridXYZ[3 * p + 2];
			}
		}
		std::string text = "analytic_signal_coherence_factor_method = none\n";
		if (d.cf == 1) {
			char buf[64];
			std::snprintf(buf, sizeof buf, "%.17g", static_cast<double>(d.pcf_gamma));
			text = std::string("analytic_signal_coherence_factor_method = phase_coherence_factor\n"
					"phase_coherence_factor_gamma = ") + buf + "\n";
		}
		TempParamFile f(text);
		ParameterMap pm(f.path);
		AnalyticSignalCoherenceFactorProcessor<T> cf(pm);
		if (d.mode == 0) {
			SA3DConfiguration<T> c;
			c.numElementsMux = 1024;
			c.numPulses = 1;
			fill_common(d, c.centerFrequency, c.maxFrequency, c.acquisitionTime, c.minGain, c.maxGain,
					c.propagationSpeed, c.acquisitionDelay, c.samplingFrequency, c.deadZoneM, c.valueScale);
			ArrayUtil::calculateElementPositions(d.pitch_x, d.nx, T(0), d.pitch_y, d.ny, T(0), c.txElemPos);
			ArrayUtil::calculateElementPositions(d.pitch_x, d.nx, T(0), d.pitch_y, d.ny, T(0), c.rxElemPos);
			c.activeTxElem.assign(d.active, d.active + d.num_active);
			c.activeRxElem.assign(d.active, d.active + d.num_active);
			SaftAcquisition<T> acq(rf, c.activeTxElem, d.num_samples);
			Vectorial3DT1R1SAFTProcessor<T> proc(c, acq, d.upsampling, cf, d.peak_offset);
			proc.prepare(0);
			proc.process(grid);
		} else {
			TnRnConfiguration<T> c;
			c.numElementsMux = d.nx * d.ny;
			c.numElements = d.num_elements;
			c.numPulses = 1;
			fill_common(d, c.centerFrequency, c.maxFrequency, c.acquisitionTime, c.minGain, c.maxGain,
					c.propagationSpeed, c.acquisitionDelay, c.samplingFrequency, c.deadZoneM, c.valueScale);
			ArrayUtil::calculateElementPositions(d.pitch_x, d.nx, T(0), d.pitch_y, d.ny, T(0), c.txElemPos);
			ArrayUtil::calculateElementPositions(d.pitch_x, d.nx, T(0), d.pitch_y, d.ny, T(0), c.rxElemPos);
			std::vector<T> txDelays;
			ArrayUtil::calculateTx3DFocusDelay(d.focus_x, d.focus_y, d.focus_z, c.propagationSpeed,
					c.txElemPos, d.base_element, c.numElements, txDelays);
			if (d.tx_delays_out) std::copy(txDelays.begin(), txDelays.end(), d.tx_delays_out);
			std::vector<T> apod(d.rx_apod, d.rx_apod + d.num_elements);
			MemoryTnRnAcquisition<T> acq(rf, d.num_elements, d.num_samples);
			if (d.mode == 1) {
				Vectorial3DTnRnProcessor<T> proc(c, acq, d.upsampling, cf, d.peak_offset, apod);
				proc.setTxDelays(d.focus_x, d.focus_y, d.focus_z, txDelays);
				proc.prepare(d.base_element);
				proc.process(grid);
			} else {
				SynthYVectorial3DTnRnProcessor<T> proc(c, acq, d.upsampling, cf, d.peak_offset, apod);
				proc.setTxDelays(d.focus_x, d.focus_y, d.focus_z, txDelays);
				proc.prepare(d.base_element);
				const std::size_t acqSize = static_cast<std::size_t>(d.num_elements) * d.num_samples;
				for (unsigned a = 0; a < d.num_acq; ++a) {
					acq.setData(rf + a * acqSize);
					proc.getAcqData(d.acq_y[a]);
				}
				proc.process(d.first_acq, d.last_acq, grid);
			}
		}
		for (unsigned i = 0; i < n1; ++i) {
			for (unsigned j = 0; j < n2; ++j) {
				const std::size_t p = static_cast<std::size_t>(i) * n2 + j;
				value[p] = grid(i, j).value;
				factor[p] = grid(i, j).factor;
			}
		}
		return 0;
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

template<typename T>
struct RefTwoMediumDesc {
	unsigned num_elements, num_elements_mux;
	T pitch, center_frequency, propagation_speed_1, propagation_speed_2, sampling_frequency;
	unsigned num_samples;        // samples per A-scan of every acquisition tensor
	unsigned upsampling;
	T max_fermat_block_size, peak_offset;
	unsigned signal_start_offset;
	unsigned num_acq, num_tx;    // acqDataList: num_acq tensors of (num_tx, num_elements, num_samples)
	unsigned num_steps;
	const unsigned* steps;       // num_steps x (baseElemIdx, baseElem, firstTxElem, lastTxElem)
	unsigned num_interface;
	const T* interface_xz;       // num_interface (x, z)
	const T* rx_apod;            // num_elements
	int cf;                      // 0 none, 1 PCF
	T pcf_gamma;
};

// VectorialCombinedTwoMediumImagingProcessor<T>::process on a grid of n1
// columns x n2 rows (x, z); out: n1 x n2 complex (re, im).
template<typename T>
int run_two_medium(const RefTwoMediumDesc<T>* dp, const T* rf, const T* gridXZ, unsigned n1, unsigned n2, T* out)
{
	try {
		const RefTwoMediumDesc<T>& d = *dp;
		TwoMediumSTAConfiguration<T> c;
		c.numElements = d.num_elements;
		c.numElementsMux = d.num_elements_mux;
		c.pitch = d.pitch;
		c.centerFrequency = d.center_frequency;
		c.acquisitionTime = 1e-4;
		c.minGain = 0;
		c.maxGain = 0;
		c.propagationSpeed1 = d.propagation_speed_1;
		c.propagationSpeed2 = d.propagation_speed_2;
		c.acquisitionDelay = 0;
		c.samplingFrequency = d.sampling_frequency;
		c.deadZoneM = 0;
		std::vector<Tensor3<T>> acqDataList(d.num_acq);
		const std::size_t acqSize = static_cast<std::size_t>(d.num_tx) * d.num_elements * d.num_samples;
		for (unsigned a = 0; a < d.num_acq; ++a) {
			acqDataList[a].resize(d.num_tx, d.num_elements, d.num_samples);
			std::copy(rf + a * acqSize, rf + (a + 1) * acqSize, &acqDataList[a](0, 0, 0));
		}
		std::string text = "analytic_signal_coherence_factor_method = none\n";
		if (d.cf == 1) {
			char buf[64];
			std::snprintf(buf, sizeof buf, "%.17g", static_cast<double>(d.pcf_gamma));
			text = std::string("analytic_signal_coherence_factor_method = phase_coherence_factor\n"
					"phase_coherence_factor_gamma = ") + buf + "\n";
		}
		TempParamFile f(text);
		ParameterMap pm(f.path);
		AnalyticSignalCoherenceFactorProcessor<T> cf(pm);
		VectorialCombinedTwoMediumImagingProcessor<T> proc(c, acqDataList, d.upsampling, cf, d.max_fermat_block_size,
				d.peak_offset, d.signal_start_offset);
		std::vector<typename VectorialCombinedTwoMediumImagingProcessor<T>::StepConfiguration> steps;
		for (unsigned i = 0; i < d.num_steps; ++i) {
			const unsigned* s = d.steps + 4 * i;
			steps.push_back({s[0], s[1], s[2], s[3]});
		}
		std::vector<XZ<T>> interfacePoints(d.num_interface);
		for (unsigned i = 0; i < d.num_interface; ++i) {
			interfacePoints[i].x = d.interface_xz[2 * i];
			interfacePoints[i].z = d.interface_xz[2 * i + 1];
		}
		std::vector<T> apod(d.rx_apod, d.rx_apod + d.num_elements);
		Matrix<XZ<T>> grid(n1, n2);
		for (unsigned i = 0; i < n1; ++i) {
			for (unsigned j = 0; j < n2; ++j) {
				const std::size_t p = static_cast<std::size_t>(i) * n2 + j;
				grid(i, j).x = gridXZ[2 * p];
				grid(i, j).z = gridXZ[2 * p + 1];
			}
		}
		Matrix<std::complex<T>> value(n1, n2);
		proc.process(steps, interfacePoints, apod, grid, value);
		for (unsigned i = 0; i < n1; ++i) {
			for (unsigned j = 0; j < n2; ++j) {
				const std::size_t p = static_cast<std::size_t>(i) * n2 + j;
				out[2 * p] = value(i, j).real();
				out[2 * p + 1] = value(i, j).imag();
			}
		}
		return 0;
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

}  // namespace

extern "C" {
const char* ref_last_error(void) { return g_err.c_str(); }
int ref_process_f32(const RefDesc<float>* d, const float* rf, const float* grid, unsigned n1, unsigned n2, float* value, float* factor)
{
	return run<float>(d, rf, grid, n1, n2, value, factor);
}
int ref_process_f64(const RefDesc<double>* d, const double* rf, const double* grid, unsigned n1, unsigned n2, double* value, double* factor)
{
	return run<double>(d, rf, grid, n1, n2, value, factor);
}
int ref_single_f32(const RefSingleDesc<float>* d, const float* rf, const float* grid, unsigned n1, unsigned n2, float* value, float* factor)
{
	return run_single<float>(d, rf, grid, n1, n2, value, factor);
}
int ref_single_f64(const RefSingleDesc<double>* d, const double* rf, const double* grid, unsigned n1, unsigned n2, double* value, double* factor)
{
	return run_single<double>(d, rf, grid, n1, n2, value, factor);
}
int ref_two_medium_f32(const RefTwoMediumDesc<float>* d, const float* rf, const float* grid, unsigned n1, unsigned n2,
		float* out)
{
	return run_two_medium<float>(d, rf, grid, n1, n2, out);
}
int ref_two_medium_f64(const RefTwoMediumDesc<double>* d, const double* rf, const double* grid, unsigned n1, unsigned n2,
		double* out)
{
	return run_two_medium<double>(d, rf, grid, n1, n2, out);
}
// The reference's WindowFunction::get (src/util/WindowFunction.h:237-289) for
// one description ("blackman", "trapezoidal 3 4 5", ...) and size, in float
// (the apodization type of the float processors). Returns -1 with the
// reference's exception message on an invalid description.
int ref_window_f32(const char* description, unsigned size, float* out)
{
	try {
		std::vector<float> w;
		Lab::WindowFunction::get<float>(description, size, w);
		if (w.size() != size) throw std::runtime_error("window size mismatch");
		std::copy(w.begin(), w.end(), out);
		return 0;
	} catch (std::exception& e) {
		g_err = e.what();
		return -1;
	}
}
}
