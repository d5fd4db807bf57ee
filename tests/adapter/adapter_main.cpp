// Compiles the drop-in processors of include/usgb_sta_processor.hpp and
// include/usgb_single_processor.hpp inside the reference's own headers and
// runs them through the reference's plugin interface
// (ArrayProcessor::prepare/process, setTxDelays, getAcqData). Prints one line
// per case.
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
#include "Tensor3.h"
#include "TnRnAcquisition.h"
#include "TnRnConfiguration.h"
#include "TwoMediumSTAConfiguration.h"
#include "XZ.h"
#include "Util.h"
#include "XYZValueFactor.h"
#include "usgb_single_processor.hpp"
#include "usgb_two_medium_processor.hpp"
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

class ZeroTnRnAcquisition : public TnRnAcquisition<float> {
public:
	ZeroTnRnAcquisition(unsigned n, unsigned ns) : n_(n), ns_(ns) {}
	void execute(AcquisitionDataType& m) override
	{
		m.resize(n_, ns_);
		for (auto& v : m) v = 0.0f;
	}
private:
	unsigned n_, ns_;
};

static void matrix_positions(std::vector<XY<float>>& pos)
{
	ArrayUtil::calculateElementPositions(0.3e-3f, 4U, 0.0f, 0.3e-3f, 4U, 0.0f, pos);
}

static TnRnConfiguration<float> tnrn_config(float deadZone)
{
	TnRnConfiguration<float> c;
	c.numElementsMux = 16;
	c.numElements = 8;
	c.numPulses = 1;
	c.centerFrequency = 5e6f;
	c.maxFrequency = 10e6f;
	c.acquisitionTime = 1e-4f;
	c.minGain = c.maxGain = 0;
	c.propagationSpeed = 1540.0f;
	c.acquisitionDelay = 0;
	c.samplingFrequency = 40e6f;
	c.deadZoneM = deadZone;
	c.valueScale = 1;
	matrix_positions(c.txElemPos);
	matrix_positions(c.rxElemPos);
	return c;
}

static void fill_grid(Matrix<XYZValueFactor<float>>& grid)
{
	for (unsigned i = 0; i < grid.n1(); ++i)
		for (unsigned j = 0; j < grid.n2(); ++j) { grid(i, j).x = 1e-3f * i; grid(i, j).z = 5e-3f + 1e-3f * j; }
}

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
	// Single-term 3D processors.
	run_case("saft_frame", [&] {
		SA3DConfiguration<float> c;
		c.numElementsMux = 16;
		c.numPulses = 1;
		c.centerFrequency = 5e6f;
		c.maxFrequency = 10e6f;
		c.acquisitionTime = 1e-4f;
		c.minGain = c.maxGain = 0;
		c.propagationSpeed = 1540.0f;
		c.acquisitionDelay = 0;
		c.samplingFrequency = 40e6f;
		c.deadZoneM = 0;
		c.valueScale = 1;
		matrix_positions(c.txElemPos);
		matrix_positions(c.rxElemPos);
		for (unsigned e = 0; e < 16; e += 2) {
			c.activeTxElem.push_back(e);
			c.activeRxElem.push_back(e);
		}
		ZeroAcquisition acq(1, 256);
		Vectorial3DT1R1SAFTGB300Processor p(c, acq, 4, noCF, 0.0f);
		Matrix<XYZValueFactor<float>> grid(4, 4);
		fill_grid(grid);
		p.prepare(0);
		p.process(grid);
	});
	run_case("tnrn_apod", [&] {
		auto c = tnrn_config(0.0f);
		ZeroTnRnAcquisition acq(8, 256);
		Vectorial3DTnRnGB300Processor p(c, acq, 4, noCF, 0.0f, std::vector<float>(7, 1.0f));
	});
	run_case("tnrn_no_delays", [&] {
		auto c = tnrn_config(0.0f);
		ZeroTnRnAcquisition acq(8, 256);
		Vectorial3DTnRnGB300Processor p(c, acq, 4, noCF, 0.0f, apod);
		p.prepare(0);
	});
	run_case("tnrn_dead_zone", [&] {
		auto c = tnrn_config(0.05f);
		ZeroTnRnAcquisition acq(8, 256);
		Vectorial3DTnRnGB300Processor p(c, acq, 4, noCF, 0.0f, apod);
		std::vector<float> delays;
		ArrayUtil::calculateTx3DFocusDelay(0.0f, 0.0f, -5e-3f, c.propagationSpeed, c.txElemPos, 0U, 8U, delays);
		p.setTxDelays(0.0f, 0.0f, -5e-3f, delays);
		Matrix<XYZValueFactor<float>> grid(4, 4);
		p.prepare(0);
		p.process(grid);
	});
	run_case("tnrn_frame", [&] {
		auto c = tnrn_config(0.0f);
		ZeroTnRnAcquisition acq(8, 256);
		Vectorial3DTnRnGB300Processor p(c, acq, 4, noCF, 0.0f, apod);
		std::vector<float> delays;
		ArrayUtil::calculateTx3DFocusDelay(0.0f, 0.0f, -5e-3f, c.propagationSpeed, c.txElemPos, 0U, 8U, delays);
		p.setTxDelays(0.0f, 0.0f, -5e-3f, delays);
		Matrix<XYZValueFactor<float>> grid(4, 4);
		fill_grid(grid);
		p.prepare(0);
		p.process(grid);
	});
	run_case("synthy_frame", [&] {
		auto c = tnrn_config(0.0f);
		ZeroTnRnAcquisition acq(8, 256);
		SynthYVectorial3DTnRnGB300Processor p(c, acq, 4, noCF, 0.0f, apod, 4);
		std::vector<float> delays;
		ArrayUtil::calculateTx3DFocusDelay(0.0f, 0.0f, -5e-3f, c.propagationSpeed, c.txElemPos, 0U, 8U, delays);
		p.setTxDelays(0.0f, 0.0f, -5e-3f, delays);
		p.prepare(0);
		for (int a = 0; a < 3; ++a) p.getAcqData(1e-4f * a);
		Matrix<XYZValueFactor<float>> grid(4, 4);
		fill_grid(grid);
		p.process(0, 2, grid);
		if (grid(0, 0).y != 1e-4f) throw std::runtime_error("center y not written");
	});
	// Two-medium imaging.
	auto two_medium = [&](const char* name, unsigned firstTx, unsigned lastTx, std::size_t nIf) {
		run_case(name, [&] {
			TwoMediumSTAConfiguration<float> c;
			c.numElements = 8;
			c.numElementsMux = 16;
			c.pitch = 0.6e-3f;
			c.centerFrequency = 5e6f;
			c.acquisitionTime = 1e-4f;
			c.minGain = c.maxGain = 0;
			c.propagationSpeed1 = 1480.0f;
			c.propagationSpeed2 = 2700.0f;
			c.acquisitionDelay = 0;
			c.samplingFrequency = 20e6f;
			c.deadZoneM = 0;
			std::vector<Tensor3<float>> acq(2);
			for (auto& t : acq) {
				t.resize(lastTx - firstTx + 1, 8, 400);
				for (auto& v : t) v = 0.0f;
			}
			VectorialCombinedTwoMediumImagingGB300Processor p(c, acq, 4, noCF, 2.0f, 1.5f, 0);
			std::vector<VectorialCombinedTwoMediumImagingGB300Processor::StepConfiguration> steps = {
				{0, 0, firstTx, lastTx}, {1, 8, firstTx, lastTx}};
			std::vector<XZ<float>> iface;
			for (std::size_t i = 0; i < nIf; ++i) iface.push_back(XZ<float>(-5e-3f + 1e-4f * i, 8e-3f));
			std::vector<float> apodTm(8, 1.0f);
			Matrix<XZ<float>> grid(4, 8);
			for (unsigned i = 0; i < 4; ++i)
				for (unsigned j = 0; j < 8; ++j) { grid(i, j).x = 1e-3f * i; grid(i, j).z = 6e-3f + 1e-3f * j; }
			Matrix<std::complex<float>> value(4, 8);
			p.process(steps, iface, apodTm, grid, value);
		});
	};
	two_medium("two_medium_frame", 0, 7, 100);
	two_medium("two_medium_onetx_frame", 3, 3, 100);
	return 0;
}
