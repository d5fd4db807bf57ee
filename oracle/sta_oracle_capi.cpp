// C entry points of the CPU oracle (test infrastructure only; see
// sta_oracle.hpp). Loaded by tests/ and by bench.py's CPU-baseline leg through
// ctypes. Every function returns 0 on success and -1 on a rejected input, with
// the message available from orc_last_error().
#include <cstring>
#include <string>

#include "sta_oracle.hpp"

namespace {
thread_local std::string g_err;

template<typename T>
struct CDesc {
	unsigned num_tx, num_rx, num_samples, upsampling;
	T sampling_frequency, propagation_speed, center_frequency, peak_offset, dead_zone_m;
	const T* tx_xy;
	const T* rx_xy;
	const T* rx_apod;
	int cf;
	T pcf_gamma, scf_p;
	int real_path;
	int nthreads;
};

template<typename T>
orc::StaDesc<T> to_desc(const CDesc<T>* c)
{
	orc::StaDesc<T> d;
	d.numTx = c->num_tx;
	d.numRx = c->num_rx;
	d.numSamples = c->num_samples;
	d.upsampling = c->upsampling;
	d.samplingFrequency = c->sampling_frequency;
	d.propagationSpeed = c->propagation_speed;
	d.centerFrequency = c->center_frequency;
	d.peakOffset = c->peak_offset;
	d.deadZoneM = c->dead_zone_m;
	d.txXY = c->tx_xy;
	d.rxXY = c->rx_xy;
	d.rxApod = c->rx_apod;
	d.cf = c->cf;
	d.pcfGamma = c->pcf_gamma;
	d.scfP = c->scf_p;
	d.realPath = c->real_path != 0;
	d.nthreads = c->nthreads;
	return d;
}

template<typename T>
int process(const CDesc<T>* c, const T* rf, const T* grid, std::size_t npix, T* value, T* factor, T* signalsOut)
{
	try {
		const orc::StaDesc<T> d = to_desc(c);
		const unsigned U = d.realPath ? 4U : d.upsampling;
		const unsigned L = d.numSamples * U;
		std::vector<std::complex<T>> analytic;
		std::vector<T> real;
		if (d.realPath) {
			orc::prepare_signals<T>(d, rf, nullptr, &real);
			if (signalsOut) std::memcpy(signalsOut, real.data(), real.size() * sizeof(T));
		} else {
			orc::prepare_signals<T>(d, rf, &analytic, nullptr);
			if (signalsOut) std::memcpy(signalsOut, analytic.data(), analytic.size() * sizeof(std::complex<T>));
		}
		if (grid && npix) {
			orc::delay_and_sum<T>(d, analytic.data(), real.data(), L, grid, npix, value, factor);
		}
		return 0;
	} catch (const std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

template<typename T>
int das_only(const CDesc<T>* c, const T* signals, const T* grid, std::size_t npix, T* value, T* factor)
{
	try {
		const orc::StaDesc<T> d = to_desc(c);
		const unsigned U = d.realPath ? 4U : d.upsampling;
		const unsigned L = d.numSamples * U;
		if (d.realPath) {
			orc::delay_and_sum<T>(d, nullptr, signals, L, grid, npix, value, factor);
		} else {
			orc::delay_and_sum<T>(d, reinterpret_cast<const std::complex<T>*>(signals), nullptr, L, grid, npix, value, factor);
		}
		return 0;
	} catch (const std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

template<typename T>
struct CSingleDesc {
	int mode;
	unsigned num_signals, num_samples, upsampling;
	T sampling_frequency, propagation_speed, center_frequency, peak_offset, dead_zone_m;
	const T* tx_xy;
	const T* rx_xy;
	const T* rx_apod;
	T focus_x, focus_y, focus_z, first_tx_delay;
	unsigned num_acq;
	const T* acq_y;
	int cf;
	T pcf_gamma, scf_p;
	int nthreads;
};

template<typename T>
int single(const CSingleDesc<T>* c, const T* rf, const T* grid, std::size_t npix, T* value, T* factor, T* signalsOut)
{
	try {
		orc::SingleDesc<T> d;
		d.mode = c->mode;
		d.numSignals = c->num_signals;
		d.numSamples = c->num_samples;
		d.upsampling = c->upsampling;
		d.samplingFrequency = c->sampling_frequency;
		d.propagationSpeed = c->propagation_speed;
		d.centerFrequency = c->center_frequency;
		d.peakOffset = c->peak_offset;
		d.deadZoneM = c->dead_zone_m;
		d.txXY = c->tx_xy;
		d.rxXY = c->rx_xy;
		d.rxApod = c->rx_apod;
		d.focusX = c->focus_x;
		d.focusY = c->focus_y;
		d.focusZ = c->focus_z;
		d.firstTxDelay = c->first_tx_delay;
		d.numAcq = (c->mode == orc::SINGLE_SYNTH_Y_TNRN) ? c->num_acq : 1U;
		d.acqY = c->acq_y;
		d.cf = c->cf;
		d.pcfGamma = c->pcf_gamma;
		d.scfP = c->scf_p;
		d.nthreads = c->nthreads;
		if (d.numSignals == 0 || d.numAcq == 0) throw std::invalid_argument("no signals");
		if (d.mode != orc::SINGLE_T1R1_SAFT && !d.rxApod) throw std::invalid_argument("missing rx apodization");
		std::vector<std::complex<T>> analytic;
		orc::prepare_single<T>(d, rf, analytic);
		if (signalsOut) std::memcpy(signalsOut, analytic.data(), analytic.size() * sizeof(std::complex<T>));
		if (grid && npix) {
			orc::single_term_das<T>(d, analytic.data(), d.numSamples * d.upsampling, grid, npix, value, factor);
		}
		return 0;
	} catch (const std::exception& e) {
		g_err = e.what();
		return -1;
	}
}

template<typename T>
struct CTwoMediumDesc {
	unsigned num_elements, num_elements_mux;
	T pitch, center_frequency, propagation_speed_1, propagation_speed_2, sampling_frequency;
	unsigned num_samples, upsampling;
	T max_fermat_block_size, peak_offset;
	unsigned signal_start_offset;
	unsigned num_acq, num_tx, num_steps;
	const unsigned* steps;
	unsigned num_interface;
	const T* interface_xz;
	const T* rx_apod;
	int cf;
	T pcf_gamma;
	int nthreads;
};

template<typename T>
int two_medium(const CTwoMediumDesc<T>* c, const T* rf, const T* grid, unsigned ncols, unsigned nrows, T* out)
{
	try {
		orc::TwoMediumDesc<T> d;
		d.numElements = c->num_elements;
		d.numElementsMux = c->num_elements_mux;
		d.pitch = c->pitch;
		d.centerFrequency = c->center_frequency;
		d.c1 = c->propagation_speed_1;
		d.c2 = c->propagation_speed_2;
		d.samplingFrequency = c->sampling_frequency;
		d.numSamples = c->num_samples;
		d.upsampling = c->upsampling;
		d.maxFermatBlockSize = c->max_fermat_block_size;
		d.peakOffset = c->peak_offset;
		d.signalStartOffset = c->signal_start_offset;
		d.numAcq = c->num_acq;
		d.numTx = c->num_tx;
		d.numSteps = c->num_steps;
		d.steps = c->steps;
		d.numInterface = c->num_interface;
		d.interfaceXZ = c->interface_xz;
		d.rxApod = c->rx_apod;
		d.cf = c->cf;
		d.pcfGamma = c->pcf_gamma;
		d.nthreads = c->nthreads;
		orc::two_medium_process<T>(d, rf, grid, ncols, nrows, reinterpret_cast<std::complex<T>*>(out));
		return 0;
	} catch (const std::exception& e) {
		g_err = e.what();
		return -1;
	}
}
}  // namespace

extern "C" {

const char* orc_last_error(void) { return g_err.c_str(); }

unsigned orc_next_fast_even_size(unsigned n) { return orc::next_fast_even_size(n); }
unsigned orc_hilbert_fft_size(unsigned n) { return orc::hilbert_fft_size(n); }

// Full processor: signal preparation then delay-and-sum. signals_out (optional)
// receives the analytic tensor (interleaved re/im, tx-major) or the real tensor.
int orc_process_f32(const CDesc<float>* d, const float* rf, const float* grid, std::size_t npix,
		float* value, float* factor, float* signals_out)
{
	return process<float>(d, rf, grid, npix, value, factor, signals_out);
}
int orc_process_f64(const CDesc<double>* d, const double* rf, const double* grid, std::size_t npix,
		double* value, double* factor, double* signals_out)
{
	return process<double>(d, rf, grid, npix, value, factor, signals_out);
}

// Delay-and-sum only, on given prepared signals.
int orc_das_f32(const CDesc<float>* d, const float* signals, const float* grid, std::size_t npix, float* value, float* factor)
{
	return das_only<float>(d, signals, grid, npix, value, factor);
}
int orc_das_f64(const CDesc<double>* d, const double* signals, const double* grid, std::size_t npix, double* value, double* factor)
{
	return das_only<double>(d, signals, grid, npix, value, factor);
}

// Single-term 3D processors (T1R1 SAFT, TnRn, synthetic-y TnRn): preparation
// of num_acq * num_signals A-scans, then the single-term delay-and-sum.
int orc_single_f32(const CSingleDesc<float>* d, const float* rf, const float* grid, std::size_t npix,
		float* value, float* factor, float* signals_out)
{
	return single<float>(d, rf, grid, npix, value, factor, signals_out);
}
int orc_single_f64(const CSingleDesc<double>* d, const double* rf, const double* grid, std::size_t npix,
		double* value, double* factor, double* signals_out)
{
	return single<double>(d, rf, grid, npix, value, factor, signals_out);
}

// Two-medium imaging (VectorialCombinedTwoMediumImagingProcessor): rf =
// num_acq x num_tx x num_elements x num_samples, grid = ncols x nrows (x, z),
// out = ncols x nrows complex (re, im).
int orc_two_medium_f32(const CTwoMediumDesc<float>* d, const float* rf, const float* grid, unsigned ncols, unsigned nrows,
		float* out)
{
	return two_medium<float>(d, rf, grid, ncols, nrows, out);
}
int orc_two_medium_f64(const CTwoMediumDesc<double>* d, const double* rf, const double* grid, unsigned ncols,
		unsigned nrows, double* out)
{
	return two_medium<double>(d, rf, grid, ncols, nrows, out);
}

// Building blocks, for the golden-vector tests.
int orc_interp_taps_f64(unsigned U, double halfTransition, double* taps, unsigned cap, unsigned* n)
{
	try {
		auto t = orc::interpolator_taps<double>(U, halfTransition);
		*n = static_cast<unsigned>(t.size());
		if (t.size() > cap) { g_err = "capacity"; return -1; }
		std::copy(t.begin(), t.end(), taps);
		return 0;
	} catch (const std::exception& e) { g_err = e.what(); return -1; }
}
int orc_interp_taps_f32(unsigned U, float halfTransition, float* taps, unsigned cap, unsigned* n)
{
	try {
		auto t = orc::interpolator_taps<float>(U, halfTransition);
		*n = static_cast<unsigned>(t.size());
		if (t.size() > cap) { g_err = "capacity"; return -1; }
		std::copy(t.begin(), t.end(), taps);
		return 0;
	} catch (const std::exception& e) { g_err = e.what(); return -1; }
}
int orc_interp4x_taps_f64(double* taps)
{
	auto t = orc::interpolator4x_taps_double();
	std::copy(t.begin(), t.end(), taps);
	return static_cast<int>(t.size());
}
int orc_upsample_f64(const double* in, unsigned len, unsigned U, const double* taps, unsigned ntaps, double* out)
{
	std::vector<double> t(taps, taps + ntaps);
	orc::upsample<double>(in, len, U, t, out);
	return 0;
}
int orc_upsample_f32(const float* in, unsigned len, unsigned U, const float* taps, unsigned ntaps, float* out)
{
	std::vector<float> t(taps, taps + ntaps);
	orc::upsample<float>(in, len, U, t, out);
	return 0;
}
int orc_hilbert_f64(const double* x, unsigned len, double* out)
{
	try {
		orc::Hilbert<double> h;
		h.analytic(x, len, reinterpret_cast<std::complex<double>*>(out));
		return 0;
	} catch (const std::exception& e) { g_err = e.what(); return -1; }
}
int orc_hilbert_f32(const float* x, unsigned len, float* out)
{
	try {
		orc::Hilbert<float> h;
		h.analytic(x, len, reinterpret_cast<std::complex<float>*>(out));
		return 0;
	} catch (const std::exception& e) { g_err = e.what(); return -1; }
}
int orc_envelope_f64(const double* x, unsigned len, unsigned count, double* out)
{
	try {
		orc::Hilbert<double> h;
		for (unsigned c = 0; c < count; ++c) h.envelope(x + static_cast<size_t>(c) * len, len, out + static_cast<size_t>(c) * len);
		return 0;
	} catch (const std::exception& e) { g_err = e.what(); return -1; }
}
int orc_envelope_f32(const float* x, unsigned len, unsigned count, float* out)
{
	try {
		orc::Hilbert<float> h;
		for (unsigned c = 0; c < count; ++c) h.envelope(x + static_cast<size_t>(c) * len, len, out + static_cast<size_t>(c) * len);
		return 0;
	} catch (const std::exception& e) { g_err = e.what(); return -1; }
}
int orc_linear_to_decibels_f32(float* data, size_t n, float min_db)
{
	orc::linear_to_decibels<float>(data, n, min_db);
	return 0;
}
int orc_linear_to_decibels_f64(double* data, size_t n, double min_db)
{
	orc::linear_to_decibels<double>(data, n, min_db);
	return 0;
}
int orc_fft_f64(const double* in, unsigned n, int sign, double* out)
{
	orc::FFT<double> f(n);
	f.execute(reinterpret_cast<const std::complex<double>*>(in), reinterpret_cast<std::complex<double>*>(out), sign);
	return 0;
}
int orc_remove_dc_f64(double* data, unsigned size, unsigned begin)
{
	try { orc::remove_dc<double>(data, size, begin); return 0; }
	catch (const std::exception& e) { g_err = e.what(); return -1; }
}
double orc_kaiser_beta_f64(double tol_dB) { return orc::kaiser_beta<double>(tol_dB); }
int orc_kaiser_size_f64(double tol_dB, double transitionWidth)
{
	try { return static_cast<int>(orc::kaiser_size<double>(tol_dB, transitionWidth)); }
	catch (const std::exception& e) { g_err = e.what(); return -1; }
}
double orc_scf_f64(const double* d, unsigned n, double p) { return orc::scf<double>(d, n, p); }
double orc_pcf_f64(const double* d, unsigned n, double gamma)
{
	std::vector<double> a, b;
	const double sigma0 = orc::kPi / std::sqrt(3.0);
	return orc::pcf<double>(reinterpret_cast<const std::complex<double>*>(d), n, gamma / sigma0, a, b);
}

}  // extern "C"
