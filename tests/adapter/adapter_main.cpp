// Compiles the drop-in processors of include/usgb_sta_processor.hpp inside the
// reference's own headers and runs them through the reference's plugin
// interface (ArrayProcessor::prepare/process). Prints one line per case.
#include <cstdio>
#include <fstream>
#include <iostream>

#include "ArrayGeometry.h"
#include "ArrayProcessor.h"
#include "CoherenceFactor.h"
#include "Exception.h"
#include "Matrix.h"
#include "SA3DConfiguration.h"
#include "STAAcquisition.h"
#include "STAConfiguration.h"
#include "Util.h"
#include "XYZValueFactor.h"
#include "usgb_sta_processor.hpp"

using namespace Lab;

class ZeroAcquisition : public STAAcquisition<float> {
public:
	ZeroAcquisition(unsigned nrx, unsigned ns) : nrx_(nrx), ns_(ns) {}
	void execute(unsigned int, AcquisitionDataType& m) override
	{
		m.resize(nrx_, ns_);
		for (auto& v : m) v = 0.0f;
	}
private:
	unsigned nrx_, ns_;
};

static STAConfiguration<float> config(float deadZone)
{
	STAConfiguration<float> c;
	c.numElementsMux = c.numElements = 8;
	c.firstTxElem = 0;
	c.lastTxElem = 7;
	c.numPulses = 1;
	c.pitch = 0.3e-3f;
	c.centerFrequency = 5e6f;
	c.maxFrequency = 10e6f;
	c.acquisitionTime = 1e-4f;
	c.minGain = c.maxGain = 0;
	c.propagationSpeed = 1540.0f;
	c.acquisitionDelay = 0;
	c.samplingFrequency = 40e6f;
	c.deadZoneM = deadZone;
	c.valueScale = 1;
	return c;
}

template<typename F>
static void run_case(const char* name, F&& f)
{
	try {
		f();
		std::printf("%s ok\n", name);
	} catch (InvalidParameterException& e) {
		std::printf("%s InvalidParameterException %s\n", name, e.what());
	} catch (InvalidValueException& e) {
		std::printf("%s InvalidValueException %s\n", name, e.what());
	} catch (InvalidStateException& e) {
		std::printf("%s InvalidStateException %s\n", name, e.what());
	} catch (std::exception& e) {
		std::printf("%s Exception %s\n", name, e.what());
	}
}

int main()
{
	std::vector<float> apod(8, 1.0f);
	AnalyticSignalCoherenceFactorProcessor<float> noCF;
	run_case("dead_zone", [&] {
		auto c = config(0.05f);  // 0.05 m -> far beyond 256 samples
		ZeroAcquisition acq(8, 256);
		VectorialSTAGB300Processor p(c, acq, 4, noCF, 0.0f, apod);
		Matrix<XYZValueFactor<float>> grid(4, 4);
		p.prepare(0);
		p.process(grid);
	});
	run_case("frame", [&] {
		auto c = config(0.0f);
		ZeroAcquisition acq(8, 256);
		VectorialSTAGB300Processor p(c, acq, 4, noCF, 0.0f, apod);
		Matrix<XYZValueFactor<float>> grid(4, 4);
		for (unsigned i = 0; i < 4; ++i)
			for (unsigned j = 0; j < 4; ++j) { grid(i, j).x = 1e-3f * i; grid(i, j).z = 5e-3f + 1e-3f * j; }
		p.prepare(0);
		p.process(grid);
		float s = 0;
		for (auto& pt : grid) s += pt.value;
		std::printf("frame sum %g\n", s);
	});
	return 0;
}
