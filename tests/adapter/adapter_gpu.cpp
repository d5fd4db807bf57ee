// Runs one frame through the drop-in processors of include/usgb_sta_processor.hpp
// (VectorialSTAGB300Processor: analytic path with or without PCF;
// DefaultSTAGB300Processor: real-RF path with or without SCF), compiled
// against stand-ins of the reference's interface types
// (standin/reference_standin.h), through the reference's plugin calls
// prepare(baseElement) and process(gridData). Test infrastructure.
//
// usage: adapter_gpu <frame.bin> <image.bin>
//   frame.bin: uint32 kind (0 vectorial, 1 default), numElements, firstTxElem,
//   lastTxElem, numSamples, upsampling, ncols, nrows, coherence (0 none,
//   1 on); float32 pitch, samplingFrequency, propagationSpeed,
//   centerFrequency, deadZoneM, peakOffset, pcfGamma, scfP; then the RF
//   ((lastTx - firstTx + 1) x numElements x numSamples float32), the grid
//   (ncols x nrows x 3 float32, x y z) and, kind 0, the receive apodization
//   (numElements float32).
//   image.bin: value then factor (ncols x nrows float32 each, column-major).
// Prints "ok" or the exception type and message.
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "reference_standin.h"
#include "usgb_sta_processor.hpp"

using namespace Lab;

namespace {

// Transmit event e (an element index) hands over its rows of the frame.
class MemoryAcquisition : public STAAcquisition<float> {
public:
	MemoryAcquisition(const std::vector<float>& rf, unsigned firstTx, unsigned numRx, unsigned ns)
		: rf_(rf), firstTx_(firstTx), numRx_(numRx), ns_(ns) {}
	void execute(unsigned int txElement, AcquisitionDataType& m) override
	{
		m.resize(numRx_, ns_);
		const float* src = rf_.data() + static_cast<size_t>(txElement - firstTx_) * numRx_ * ns_;
		std::copy(src, src + static_cast<size_t>(numRx_) * ns_, m.data());
	}
private:
	const std::vector<float>& rf_;
	unsigned firstTx_, numRx_, ns_;
};

template<typename T>
void read(std::ifstream& in, T* p, size_t n)
{
	in.read(reinterpret_cast<char*>(p), static_cast<std::streamsize>(n * sizeof(T)));
	if (!in) throw std::runtime_error("short input file");
}

}  // namespace

int main(int argc, char** argv)
{
	if (argc != 3) {
		std::fprintf(stderr, "usage: adapter_gpu <frame.bin> <image.bin>\n");
		return 2;
	}
	try {
		std::ifstream in(argv[1], std::ios::binary);
		uint32_t h[9];
		float f[8];
		read(in, h, 9);
		read(in, f, 8);
		const unsigned kind = h[0], numElements = h[1], firstTx = h[2], lastTx = h[3], ns = h[4], U = h[5];
		const unsigned ncols = h[6], nrows = h[7], coherence = h[8];
		STAConfiguration<float> config;
		config.numElements = numElements;
		config.numElementsMux = numElements;
		config.firstTxElem = firstTx;
		config.lastTxElem = lastTx;
		config.pitch = f[0];
		config.samplingFrequency = f[1];
		config.propagationSpeed = f[2];
		config.centerFrequency = f[3];
		config.deadZoneM = f[4];
		const float peakOffset = f[5], pcfGamma = f[6], scfP = f[7];
		std::vector<float> rf(static_cast<size_t>(lastTx - firstTx + 1) * numElements * ns);
		read(in, rf.data(), rf.size());
		std::vector<float> xyz(static_cast<size_t>(ncols) * nrows * 3);
		read(in, xyz.data(), xyz.size());
		std::vector<float> apod;
		if (kind == 0) {
			apod.resize(numElements);
			read(in, apod.data(), apod.size());
		}

		Matrix<XYZValueFactor<float>> grid(ncols, nrows);
		for (unsigned i = 0; i < ncols; ++i) {
			for (unsigned j = 0; j < nrows; ++j) {
				const float* q = &xyz[(static_cast<size_t>(i) * nrows + j) * 3];
				grid(i, j).x = q[0];
				grid(i, j).y = q[1];
				grid(i, j).z = q[2];
			}
		}
		MemoryAcquisition acq(rf, firstTx, numElements, ns);
		if (kind == 0) {
			AnalyticSignalCoherenceFactorProcessor<float> cf = coherence
					? AnalyticSignalCoherenceFactorProcessor<float>(pcfGamma)
					: AnalyticSignalCoherenceFactorProcessor<float>();
			VectorialSTAGB300Processor proc(config, acq, U, cf, peakOffset, apod);
			proc.prepare(0);
			proc.process(grid);
		} else {
			CoherenceFactorProcessor<float> cf(coherence != 0);
			DefaultSTAGB300Processor proc(config, acq, cf, peakOffset, scfP);
			proc.prepare(0);
			proc.process(grid);
		}
		std::vector<float> out(2 * static_cast<size_t>(ncols) * nrows);
		const size_t n = static_cast<size_t>(ncols) * nrows;
		for (size_t p = 0; p < n; ++p) {
			out[p] = grid.data()[p].value;
			out[n + p] = grid.data()[p].factor;
		}
		std::ofstream o(argv[2], std::ios::binary);
		o.write(reinterpret_cast<const char*>(out.data()), static_cast<std::streamsize>(out.size() * sizeof(float)));
		std::cout << "ok" << std::endl;
	} catch (const InvalidValueException& e) {
		std::cout << "InvalidValueException " << e.what() << std::endl;
	} catch (const InvalidParameterException& e) {
		std::cout << "InvalidParameterException " << e.what() << std::endl;
	} catch (const InvalidStateException& e) {
		std::cout << "InvalidStateException " << e.what() << std::endl;
	} catch (const Exception& e) {
		std::cout << "Exception " << e.what() << std::endl;
	} catch (const std::exception& e) {
		std::cout << "std::exception " << e.what() << std::endl;
	}
	return 0;
}
