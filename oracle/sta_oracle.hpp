// CPU oracle for the STA/TFM delay-and-sum path of us_lab4a.
//
// TEST INFRASTRUCTURE ONLY. This is a restatement, in plain C++17, of the
// reference processors' arithmetic. It is the parity checker for the CUDA
// library and the CPU baseline that bench.py reports; the product never links,
// loads or calls it.
//
// Every function names the reference file:line it follows. TFloat is float for
// the FP32 parity target (VectorialSTAProcessor<float,...>) and double for the
// FP64 oracle (VectorialSTAProcessor<double,...>). Expressions that the
// reference evaluates in mixed float/double are evaluated the same way here.
#ifndef USGB_STA_ORACLE_HPP
#define USGB_STA_ORACLE_HPP

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <limits>
#include <stdexcept>
#include <thread>
#include <vector>

namespace orc {

constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// Sizes.
// ---------------------------------------------------------------------------

// Smallest even n' >= n whose only prime factors are 2, 3 and 5.
// Follows src/fft/FFTUtil.h:85-135 (nextFastEvenSize).
inline unsigned next_fast_even_size(unsigned n)
{
	if (n == 0) throw std::invalid_argument("n must be > 0");
	if (n & 1U) ++n;
	for (;;) {
		unsigned m = n;
		while ((m & 1U) == 0) m >>= 1;
		while (m % 3 == 0) m /= 3;
		while (m % 5 == 0) m /= 5;
		if (m == 1) return n;
		n += 2;
	}
}

// Hilbert FFT size for an A-scan of `len` samples.
// Follows src/util/HilbertEnvelope.h:152 (minPadding = 1024, at least 2048).
inline unsigned hilbert_fft_size(unsigned len)
{
	return std::max(next_fast_even_size(len + 1024U), 2048U);
}

// ---------------------------------------------------------------------------
// Parallel loop (the reference uses tbb::parallel_for over receivers and over
// grid columns; results do not depend on the partition because every output
// is computed by one thread in a fixed order).
// ---------------------------------------------------------------------------
inline void parallel_for(std::size_t n, int nthreads, const std::function<void(std::size_t, std::size_t)>& body)
{
	if (nthreads <= 1 || n < 2) {
		body(0, n);
		return;
	}
	const std::size_t nt = std::min<std::size_t>(static_cast<std::size_t>(nthreads), n);
	std::atomic<std::size_t> next{0};
	const std::size_t grain = std::max<std::size_t>(1, n / (nt * 8));
	std::vector<std::thread> pool;
	pool.reserve(nt);
	for (std::size_t t = 0; t < nt; ++t) {
		pool.emplace_back([&]() {
			for (;;) {
				const std::size_t b = next.fetch_add(grain);
				if (b >= n) break;
				body(b, std::min(n, b + grain));
			}
		});
	}
	for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------
// Complex FFT (own implementation; the reference links FFTW3, which is absent
// here). Iterative Stockham autosort, radices 4, 2, 3, 5 and a direct DFT for
// any other prime factor. Twiddles are evaluated directly in double and then
// rounded to T, so each twiddle is within half an ulp.
// sign = -1: forward (FFTW_FORWARD), sign = +1: backward (unnormalised).
// ---------------------------------------------------------------------------
template<typename T>
class FFT {
public:
	using C = std::complex<T>;

	FFT() = default;
	explicit FFT(unsigned n) { init(n); }

	void init(unsigned n)
	{
		n_ = n;
		radices_.clear();
		unsigned m = n;
		while (m % 4 == 0) { radices_.push_back(4); m /= 4; }
		while (m % 2 == 0) { radices_.push_back(2); m /= 2; }
		while (m % 3 == 0) { radices_.push_back(3); m /= 3; }
		while (m % 5 == 0) { radices_.push_back(5); m /= 5; }
		for (unsigned p = 7; m > 1; p += 2) {
			while (m % p == 0) { radices_.push_back(p); m /= p; }
		}
		// Per-stage twiddles w_{l p}^{q k}, k < l, q < p.
		tw_.clear();
		twInv_.clear();
		stageOffset_.clear();
		unsigned l = 1;
		for (unsigned p : radices_) {
			stageOffset_.push_back(static_cast<unsigned>(tw_.size()));
			for (unsigned k = 0; k < l; ++k) {
				for (unsigned q = 0; q < p; ++q) {
					const double a = -2.0 * kPi * static_cast<double>(q) * static_cast<double>(k) /
							static_cast<double>(l * p);
					tw_.emplace_back(static_cast<T>(std::cos(a)), static_cast<T>(std::sin(a)));
					twInv_.emplace_back(static_cast<T>(std::cos(a)), -static_cast<T>(std::sin(a)));
				}
			}
			l *= p;
		}
		work_.assign(n, C(0));
	}

	unsigned size() const { return n_; }

	// out may alias in.
	void execute(const C* in, C* out, int sign)
	{
		bufA_.assign(in, in + n_);
		bufB_.resize(n_);
		C* x = bufA_.data();
		C* y = bufB_.data();
		unsigned l = 1;
		for (std::size_t s = 0; s < radices_.size(); ++s) {
			const unsigned p = radices_[s];
			const unsigned m = n_ / (l * p);
			const C* tw = (sign > 0 ? twInv_.data() : tw_.data()) + stageOffset_[s];
			switch (p) {
			case 2: stage<2>(x, y, tw, l, m, sign); break;
			case 3: stage<3>(x, y, tw, l, m, sign); break;
			case 4: stage<4>(x, y, tw, l, m, sign); break;
			case 5: stage<5>(x, y, tw, l, m, sign); break;
			default: stage_generic(x, y, tw, p, l, m, sign); break;
			}
			std::swap(x, y);
			l *= p;
		}
		std::copy(x, x + n_, out);
	}

private:
	// One Stockham stage of radix P: y[k + l q + l P r] = DFT_P over q of
	// x[k + l (r + q m)] * w_{lP}^{q k}.
	template<unsigned P>
	static void stage(const C* x, C* y, const C* tw, unsigned l, unsigned m, int sign)
	{
		for (unsigned r = 0; r < m; ++r) {
			for (unsigned k = 0; k < l; ++k) {
				C v[P];
				v[0] = x[k + l * r];
				for (unsigned q = 1; q < P; ++q) v[q] = x[k + l * (r + q * m)] * tw[k * P + q];
				butterfly(v, P, sign);
				for (unsigned q = 0; q < P; ++q) y[k + l * q + l * P * r] = v[q];
			}
		}
	}

	static void stage_generic(const C* x, C* y, const C* tw, unsigned p, unsigned l, unsigned m, int sign)
	{
		std::vector<C> v(p);
		for (unsigned r = 0; r < m; ++r) {
			for (unsigned k = 0; k < l; ++k) {
				v[0] = x[k + l * r];
				for (unsigned q = 1; q < p; ++q) v[q] = x[k + l * (r + q * m)] * tw[k * p + q];
				butterfly(v.data(), p, sign);
				for (unsigned q = 0; q < p; ++q) y[k + l * q + l * p * r] = v[q];
			}
		}
	}

	static void butterfly(C* v, unsigned p, int sign)
	{
		const T s = static_cast<T>(sign);
		switch (p) {
		case 2: {
			const C a = v[0], b = v[1];
			v[0] = a + b; v[1] = a - b;
			return;
		}
		case 3: {
			const T c1 = static_cast<T>(-0.5);
			const T s1 = static_cast<T>(0.86602540378443864676) * s;  // sin(2pi/3) * sign
			const C a = v[0], b = v[1], c = v[2];
			const C t1 = b + c;
			const C t2 = a + c1 * t1;
			const C t3 = (b - c) * C(0, s1);
			v[0] = a + t1; v[1] = t2 + t3; v[2] = t2 - t3;
			return;
		}
		case 4: {
			const C a = v[0], b = v[1], c = v[2], d = v[3];
			const C t0 = a + c, t1 = a - c, t2 = b + d;
			const C t3 = (b - d) * C(0, s);  // multiply by +-i
			v[0] = t0 + t2; v[2] = t0 - t2;
			v[1] = t1 + t3; v[3] = t1 - t3;
			return;
		}
		case 5: {
			const T c1 = static_cast<T>(0.30901699437494742410);   // cos(2pi/5)
			const T c2 = static_cast<T>(-0.80901699437494742410);  // cos(4pi/5)
			const T s1 = static_cast<T>(0.95105651629515357212) * s;
			const T s2 = static_cast<T>(0.58778525229247312917) * s;
			const C a = v[0];
			const C b1 = v[1] + v[4], b2 = v[2] + v[3];
			const C d1 = v[1] - v[4], d2 = v[2] - v[3];
			const C r1 = a + c1 * b1 + c2 * b2;
			const C r2 = a + c2 * b1 + c1 * b2;
			const C i1 = C(0, 1) * (s1 * d1 + s2 * d2);
			const C i2 = C(0, 1) * (s2 * d1 - s1 * d2);
			v[0] = a + b1 + b2;
			v[1] = r1 + i1; v[4] = r1 - i1;
			v[2] = r2 + i2; v[3] = r2 - i2;
			return;
		}
		default: {
			std::vector<C> out(p, C(0));
			for (unsigned k = 0; k < p; ++k) {
				for (unsigned j = 0; j < p; ++j) {
					const double a = static_cast<double>(sign) * 2.0 * kPi *
							static_cast<double>((static_cast<unsigned long long>(j) * k) % p) / static_cast<double>(p);
					out[k] += v[j] * C(static_cast<T>(std::cos(a)), static_cast<T>(std::sin(a)));
				}
			}
			std::copy(out.begin(), out.end(), v);
			return;
		}
		}
	}

	unsigned n_ = 0;
	std::vector<unsigned> radices_;
	std::vector<unsigned> stageOffset_;
	std::vector<C> tw_, twInv_;
	std::vector<C> work_;
	std::vector<C> bufA_, bufB_;
};

// ---------------------------------------------------------------------------
// Kaiser window helpers. Follow src/util/KaiserWindow.h:45-93.
// ---------------------------------------------------------------------------
template<typename T>
T kaiser_beta(T tolerance_dB)
{
	T beta;
	if (tolerance_dB > 50) {
		beta = 0.1102 * (tolerance_dB - 8.7);
	} else if (tolerance_dB > 21) {
		const double k = tolerance_dB - 21.0;
		beta = 0.5842 * std::pow(k, 0.4) + 0.07886 * k;
	} else {
		beta = 0.0;
	}
	return beta;
}

template<typename T>
unsigned kaiser_size(T tolerance_dB, T transitionWidth)
{
	const double size = std::ceil((tolerance_dB - 7.95) / (2.285 * transitionWidth * kPi) + 1.0);
	if (size < 2.0 || size >= static_cast<double>(std::numeric_limits<unsigned>::max())) {
		throw std::invalid_argument("invalid Kaiser window size");
	}
	return static_cast<unsigned>(size);
}

inline double bessel_i0(double x) { return std::cyl_bessel_i(0.0, x); }
inline float bessel_i0(float x) { return std::cyl_bessel_if(0.0f, x); }

template<typename T>
void kaiser_window(unsigned size, T beta, std::vector<T>& w)
{
	if (size < 2) throw std::invalid_argument("invalid Kaiser window size");
	w.resize(size);
	const T c1 = 2 / static_cast<T>(size - 1U);
	const T c2 = 1 / bessel_i0(beta);
	for (unsigned n = 0; n < size; ++n) {
		const T k = c1 * n - 1;
		T x = 1 - k * k;
		if (x < 0.0) x = 0.0;
		w[n] = c2 * bessel_i0(static_cast<T>(beta * std::sqrt(x)));
	}
}

// sin(x)/x, evaluated in double (the reference passes a double argument to
// boost::math::sinc_pi; its series branch near 0 agrees with sin(x)/x to
// within rounding).
inline double sinc_of(double x)
{
	if (std::abs(x) < 1.0e-5) return 1.0 - x * x / 6.0;
	return std::sin(x) / x;
}

// Low-pass FIR of the upsampler: Kaiser-windowed sinc, tolerance 1e-4, length
// rounded up to a multiple of 2U plus 1.
// Follows src/util/Interpolator.h:64-111 and Util::fillSequenceFromStartToEndWithSize
// (src/util/Util.h:328-345).
template<typename T>
std::vector<T> interpolator_taps(unsigned U, T halfTransitionWidth)
{
	if (U < 2 || U > 64) throw std::invalid_argument("invalid upsampling factor");
	if (halfTransitionWidth > 1) throw std::invalid_argument("invalid transition width");
	const double kaiserTolerance = 1.0e-4;
	const T tol_dB = -20.0 * std::log10(kaiserTolerance);
	const T beta = kaiser_beta<T>(tol_dB);
	const T finalTransitionWidth = (halfTransitionWidth * 2) / U;
	const unsigned windowSize = kaiser_size<T>(tol_dB, finalTransitionWidth);
	const T twoUp = 2 * U;
	const unsigned finalSize = static_cast<unsigned>(std::ceil((windowSize - 1) / twoUp) * twoUp) + 1U;

	std::vector<T> window;
	kaiser_window<T>(finalSize, beta, window);

	const T numPeriods = (finalSize - 1U) / twoUp;
	std::vector<T> x(finalSize);
	{
		const double step = static_cast<double>(numPeriods - (-numPeriods)) / (finalSize - 1U);
		x[0] = -numPeriods;
		for (unsigned i = 1; i < finalSize; ++i) x[i] = -numPeriods + i * step;
	}
	std::vector<T> taps(finalSize);
	for (unsigned i = 0; i < finalSize; ++i) {
		taps[i] = static_cast<T>(sinc_of(kPi * x[i]));
	}
	for (unsigned i = 0; i < finalSize; ++i) taps[i] *= window[i];
	return taps;
}

// Fixed 4x low-pass FIR of the real-RF path, regenerated from the recipe
// stated in src/util/Interpolator4X.h:56-66 (Octave: n = 10 periods * 8,
// kaiser(n + 1, beta = 5) .* sinc(linspace(-10, 10, n + 1))), in double.
inline std::vector<double> interpolator4x_taps_double()
{
	const unsigned n = 80;
	const double beta = 5.0;
	std::vector<double> h(n + 1);
	const double i0b = std::cyl_bessel_i(0.0, beta);
	for (unsigned i = 0; i <= n; ++i) {
		const double r = 2.0 * i / n - 1.0;
		double arg = 1.0 - r * r;
		if (arg < 0.0) arg = 0.0;
		const double w = std::cyl_bessel_i(0.0, beta * std::sqrt(arg)) / i0b;
		const double xv = -10.0 + 20.0 * i / n;
		const double s = (xv == 0.0) ? 1.0 : std::sin(kPi * xv) / (kPi * xv);
		h[i] = s * w;
	}
	return h;
}

// Upsampling by zero stuffing and linear convolution with `taps`, keeping
// samples [(taps-1)/2, (taps-1)/2 + len*U) of the full convolution.
// Follows src/util/Interpolator.h:113-138; the overlap-save FFT convolution of
// src/util/FFTWFilter.h:239-289 computes this same linear convolution.
template<typename T>
void upsample(const T* in, unsigned len, unsigned U, const std::vector<T>& taps, T* out)
{
	const long ntaps = static_cast<long>(taps.size());
	const long off = (ntaps - 1) / 2;
	const long L = static_cast<long>(len) * U;
	for (long n = 0; n < L; ++n) {
		const long j = n + off;  // index into the full convolution
		T acc = 0;
		// out[n] = sum_m taps[m] * up[j - m], up[i] = in[i / U] if i % U == 0:
		// m runs over j % U, j % U + U, ... (ascending), source index (j - m) / U.
		const long m0 = j % U;
		long src = (j - m0) / U;
		// Skip taps whose source lies past the end of the input.
		long m = m0;
		if (src >= static_cast<long>(len)) {
			const long skip = src - static_cast<long>(len) + 1;
			m += skip * U;
			src -= skip;
		}
		for (; m < ntaps && src >= 0; m += U, --src) acc += taps[m] * in[src];
		out[n] = acc;
	}
}

// Subtract the mean of data[beginOffset, size) from all `size` samples.
// Follows src/util/Util.h:1009-1018.
template<typename T>
void remove_dc(T* data, std::size_t size, std::size_t beginOffset)
{
	if (beginOffset >= size) throw std::invalid_argument("invalid beginOffset");
	T sum = 0;
	for (std::size_t i = beginOffset; i < size; ++i) sum += data[i];
	const T term = -sum / static_cast<T>(size - beginOffset);
	for (std::size_t i = 0; i < size; ++i) data[i] += term;
}

// Analytic signal by FFT: zero-pad to N, forward real FFT, halve bins 0 and
// N/2, zero bins N/2+1..N-1, backward complex FFT, scale 2/N, keep the first
// `len`. Follows src/util/HilbertEnvelope.h:142-197 and :227-251.
template<typename T>
class Hilbert {
public:
	using C = std::complex<T>;
	void analytic(const T* x, unsigned len, C* out)
	{
		if (len == 0 || len > (1U << 20)) throw std::invalid_argument("invalid Hilbert input size");
		const unsigned N = hilbert_fft_size(len);
		const unsigned M = N / 2;
		if (fft_.size() != N) {
			fft_.init(N);
			half_.init(M);
			wN_.resize(M + 1);
			for (unsigned k = 0; k <= M; ++k) {
				const double a = -2.0 * kPi * static_cast<double>(k) / N;
				wN_[k] = C(static_cast<T>(std::cos(a)), static_cast<T>(std::sin(a)));
			}
		}
		// Forward real FFT of the zero-padded signal (FFTW's r2c computes the
		// same bins): an M-point complex FFT of z[n] = x[2n] + i x[2n+1] and
		// X[k] = E[k] + W_N^k O[k], E = (Z[k] + conj Z[M-k]) / 2,
		// O = (Z[k] - conj Z[M-k]) / 2i, for k = 0..M.
		z_.assign(M, C(0));
		for (unsigned i = 0; i < len; ++i) {
			if (i & 1U) z_[i / 2] = C(z_[i / 2].real(), x[i]);
			else z_[i / 2] = C(x[i], z_[i / 2].imag());
		}
		half_.execute(z_.data(), z_.data(), -1);
		buf_.assign(N, C(0));
		for (unsigned k = 0; k <= M; ++k) {
			const C a = z_[k % M];
			const C b = std::conj(z_[(M - k) % M]);
			const C e = (a + b) * static_cast<T>(0.5);
			const C o = (a - b) * C(0, static_cast<T>(-0.5));
			buf_[k] = e + wN_[k] * o;
		}
		// HilbertEnvelope::process: halve bins 0 and N/2, zero the negative
		// frequencies (already zero), backward FFT, scale 2/N.
		buf_[0] = C(buf_[0].real() * static_cast<T>(0.5), buf_[0].imag());
		buf_[M] = C(buf_[M].real() * static_cast<T>(0.5), buf_[M].imag());
		fft_.execute(buf_.data(), buf_.data(), +1);
		const T coef = 2 / static_cast<T>(N);
		for (unsigned i = 0; i < len; ++i) out[i] = C(coef * buf_[i].real(), coef * buf_[i].imag());
	}
	// HilbertEnvelope::calculate (src/util/HilbertEnvelope.h:211-232): the
	// magnitude of the analytic signal, |coef * IFFT| (std::abs of the complex
	// value, ComplexToScaledAbsoluteOp).
	void envelope(const T* x, unsigned len, T* out)
	{
		std::vector<C> a(len);
		analytic(x, len, a.data());
		for (unsigned i = 0; i < len; ++i) out[i] = std::abs(a[i]);
	}
private:
	FFT<T> fft_, half_;
	std::vector<C> buf_, z_, wN_;
};

// ---------------------------------------------------------------------------
// Geometry. Follows src/util/Geometry.h:55-84.
// ---------------------------------------------------------------------------
template<typename T>
T distance3d_z0(T x0, T y0, T x1, T y1, T z1)
{
	const T dx = x1 - x0;
	const T dy = y1 - y0;
	return std::sqrt(dx * dx + dy * dy + z1 * z1);
}

// ---------------------------------------------------------------------------
// Coherence factors.
// ---------------------------------------------------------------------------

// Population standard deviation, two-pass. Follows src/util/Statistics.h:34-58.
template<typename T>
T std_dev(const T* d, std::size_t n)
{
	T s = 0;
	for (std::size_t i = 0; i < n; ++i) s += d[i];
	const T mean = s / n;
	T acc = 0;
	for (std::size_t i = 0; i < n; ++i) {
		const T e = d[i] - mean;
		acc += e * e;
	}
	return std::sqrt(acc / n);
}

// Phase coherence factor (Camacho et al. 2009).
// Follows src/util/CoherenceFactor.h:240-296.
template<typename T>
T pcf(const std::complex<T>* d, unsigned n, T factor, std::vector<T>& phi, std::vector<T>& phiAux)
{
	phi.resize(n);
	phiAux.resize(n);
	for (unsigned i = 0; i < n; ++i) {
		phi[i] = std::atan2(d[i].imag(), d[i].real());
		phiAux[i] = phi[i] + ((phi[i] < 0) ? T(kPi) : -T(kPi));
	}
	const T sf = std::min(std_dev(phi.data(), n), std_dev(phiAux.data(), n));
	return std::max<T>(0, 1 - factor * sf);
}

// Sign coherence factor on real values, sign(0) = +1.
// Follows src/util/CoherenceFactor.h:217-236.
template<typename T>
T scf(const T* d, unsigned size, T p)
{
	unsigned n = 0;
	int signSum = 0;
	for (unsigned i = 0; i < size; ++i) {
		if (d[i] >= 0) ++signSum; else --signSum;
		++n;
	}
	const T k = static_cast<T>(signSum) / n;
	const T m = 1 - std::sqrt(1 - k * k);
	return std::pow(std::abs(m), p);
}

// Mallart-Fink coherence factor |sum s|^2 / (N sum |s|^2). The reference has
// no such factor; this definition is the library's own.
template<typename T>
T mallart_fink_cf(const std::complex<T>* d, unsigned n)
{
	std::complex<T> s(0);
	T e = 0;
	for (unsigned i = 0; i < n; ++i) {
		s += d[i];
		e += std::norm(d[i]);
	}
	if (e == 0) return 0;
	return std::norm(s) / (static_cast<T>(n) * e);
}

enum CFKind { CF_NONE = 0, CF_PCF = 1, CF_SCF = 2, CF_MF = 3 };

// ---------------------------------------------------------------------------
// Whole processor.
// ---------------------------------------------------------------------------
// Util::linearToDecibels(std::vector<T>&, T minDecibels) (src/util/Util.h:600-613):
// normalize by the largest magnitude (Util::normalize, :1031-1037: nothing
// when it is 0), then 20 log10(v), or minDecibels where v <= 10^(minDecibels/20)
// (decibelsToLinear, :588-592, evaluated in T).
template<typename T>
void linear_to_decibels(T* data, std::size_t n, T minDecibels)
{
	T maxAbs = 0;
	for (std::size_t i = 0; i < n; ++i) maxAbs = std::max(maxAbs, std::abs(data[i]));
	if (maxAbs != 0) {
		const T coeff = 1 / maxAbs;
		for (std::size_t i = 0; i < n; ++i) data[i] *= coeff;
	}
	const T minVal = std::pow(T(10), minDecibels * T(0.05));
	for (std::size_t i = 0; i < n; ++i) {
		data[i] = (data[i] <= minVal) ? minDecibels : T(20) * std::log10(data[i]);
	}
}

template<typename T>
struct StaDesc {
	unsigned numTx = 0;          // active transmit elements
	unsigned numRx = 0;          // receive elements
	unsigned numSamples = 0;     // samples per A-scan at fs
	unsigned upsampling = 1;     // 1 = no upsampling
	T samplingFrequency = 0;
	T propagationSpeed = 0;
	T centerFrequency = 0;
	T peakOffset = 0;
	T deadZoneM = 0;
	const T* txXY = nullptr;     // numTx (x, y) pairs, metres
	const T* rxXY = nullptr;     // numRx (x, y) pairs, metres
	const T* rxApod = nullptr;   // numRx weights (analytic path)
	int cf = CF_NONE;
	T pcfGamma = 1;
	T scfP = 1;
	bool realPath = false;       // DefaultSTAProcessor semantics
	int nthreads = 1;
};

// deadZoneSamplesUp, evaluated as in src/user/processor/VectorialSTAProcessor.h:138.
template<typename T>
unsigned dead_zone_samples(const StaDesc<T>& d, unsigned U)
{
	return static_cast<unsigned>((U * d.samplingFrequency) * 2.0 * d.deadZoneM / d.propagationSpeed);
}

// Signal preparation of every A-scan into `tensor` (numTx * numRx * L).
// Analytic path: follows src/user/processor/VectorialSTAProcessor.h:169-235.
// Real path: follows src/user/processor/DefaultSTAProcessor.h:121-156.
template<typename T>
void prepare_signals(const StaDesc<T>& d, const T* rf, std::vector<std::complex<T>>* analytic, std::vector<T>* real)
{
	const unsigned U = d.realPath ? 4U : d.upsampling;
	const unsigned L = d.numSamples * U;
	const unsigned dz = dead_zone_samples(d, U);
	if (dz >= L) throw std::invalid_argument("invalid dead zone");
	std::vector<T> taps;
	if (d.realPath) {
		const std::vector<double> h = interpolator4x_taps_double();
		taps.assign(h.begin(), h.end());
	} else if (U > 1) {
		taps = interpolator_taps<T>(U, static_cast<T>(0.2));
	}
	const std::size_t numSig = static_cast<std::size_t>(d.numTx) * d.numRx;
	if (analytic) analytic->assign(numSig * L, std::complex<T>(0));
	if (real) real->assign(numSig * L, T(0));
	parallel_for(numSig, d.nthreads, [&](std::size_t b, std::size_t e) {
		std::vector<T> sig(L);
		Hilbert<T> hil;
		for (std::size_t a = b; a < e; ++a) {
			const T* src = rf + a * d.numSamples;
			if (U > 1) {
				upsample<T>(src, d.numSamples, U, taps, sig.data());
			} else {
				std::copy(src, src + d.numSamples, sig.begin());
			}
			remove_dc<T>(sig.data(), L, dz);
			if (d.realPath) {
				std::copy(sig.begin(), sig.end(), real->begin() + a * L);
			} else {
				hil.analytic(sig.data(), L, analytic->data() + a * L);
			}
		}
	});
}

// Delay-and-sum over every tx x rx pair for each grid point, with optional
// coherence factor.
// Analytic path: follows src/user/processor/VectorialSTAProcessor.h:237-338
// (with the 3D delay of src/user/processor/Vectorial3DSTAProcessor.h:208-242;
// for y = 0 it equals distance2DY0 bit for bit).
// Real path: follows src/user/processor/DefaultSTAProcessor.h:158-223.
// gridXYZ: npix (x, y, z) triples. value/factor: npix each.
template<typename T>
void delay_and_sum(const StaDesc<T>& d, const std::complex<T>* analytic, const T* real, unsigned L,
		const T* gridXYZ, std::size_t npix, T* value, T* factor)
{
	const unsigned U = d.realPath ? 4U : d.upsampling;
	const T invCT = (d.samplingFrequency * U) / d.propagationSpeed;
	const T signalOffset = (d.samplingFrequency * U) * d.peakOffset / d.centerFrequency;
	const std::size_t numSignals = static_cast<std::size_t>(d.numTx) * d.numRx;
	T pcfFactor = 0;
	if (d.cf == CF_PCF) {
		const T sigma0 = kPi / std::sqrt(3.0);
		pcfFactor = d.pcfGamma / sigma0;
	}
	parallel_for(npix, d.nthreads, [&](std::size_t b, std::size_t e) {
		std::vector<T> txDelay(d.numTx), rxDelay(d.numRx);
		std::vector<std::complex<T>> rxSum(d.numRx);
		std::vector<T> rxSumReal(d.numRx);
		std::vector<T> phi, phiAux;
		for (std::size_t p = b; p < e; ++p) {
			const T px = gridXYZ[3 * p], py = gridXYZ[3 * p + 1], pz = gridXYZ[3 * p + 2];
			for (unsigned i = 0; i < d.numTx; ++i) {
				txDelay[i] = distance3d_z0<T>(d.txXY[2 * i], d.txXY[2 * i + 1], px, py, pz) * invCT;
			}
			for (unsigned i = 0; i < d.numRx; ++i) {
				rxDelay[i] = distance3d_z0<T>(d.rxXY[2 * i], d.rxXY[2 * i + 1], px, py, pz) * invCT;
			}
			T f = 1;
			T v;
			if (d.realPath) {
				std::fill(rxSumReal.begin(), rxSumReal.end(), T(0));
				for (unsigned tx = 0; tx < d.numTx; ++tx) {
					const T txD = txDelay[tx];
					for (unsigned rx = 0; rx < d.numRx; ++rx) {
						const T delay = signalOffset + txD + rxDelay[rx];
						const std::size_t idx = static_cast<std::size_t>(delay);
						const T k = delay - idx;
						if (idx + 1U < L) {
							const T* s = real + (static_cast<std::size_t>(tx) * d.numRx + rx) * L + idx;
							rxSumReal[rx] += (1 - k) * s[0] + k * s[1];
						}
					}
				}
				if (d.cf == CF_SCF) f = scf<T>(rxSumReal.data(), d.numRx, d.scfP);
				T acc = 0;
				for (unsigned rx = 0; rx < d.numRx; ++rx) acc += rxSumReal[rx];
				v = acc;
			} else if (d.cf == CF_NONE) {
				std::complex<T> sum(0);
				for (unsigned tx = 0; tx < d.numTx; ++tx) {
					const T txD = txDelay[tx];
					for (unsigned rx = 0; rx < d.numRx; ++rx) {
						const T delay = signalOffset + txD + rxDelay[rx];
						const std::size_t idx = static_cast<std::size_t>(delay);
						const T k = delay - idx;
						if (idx + 1U < L) {
							const std::complex<T>* s = analytic + (static_cast<std::size_t>(tx) * d.numRx + rx) * L + idx;
							sum += ((1 - k) * s[0] + k * s[1]) * d.rxApod[rx];
						}
					}
				}
				v = std::abs(sum);
			} else {
				std::fill(rxSum.begin(), rxSum.end(), std::complex<T>(0));
				for (unsigned tx = 0; tx < d.numTx; ++tx) {
					const T txD = txDelay[tx];
					for (unsigned rx = 0; rx < d.numRx; ++rx) {
						const T delay = signalOffset + txD + rxDelay[rx];
						const std::size_t idx = static_cast<std::size_t>(delay);
						const T k = delay - idx;
						if (idx + 1U < L) {
							const std::complex<T>* s = analytic + (static_cast<std::size_t>(tx) * d.numRx + rx) * L + idx;
							rxSum[rx] += ((1 - k) * s[0] + k * s[1]) * d.rxApod[rx];
						}
					}
				}
				if (d.cf == CF_PCF) {
					f = pcf<T>(rxSum.data(), d.numRx, pcfFactor, phi, phiAux);
				} else if (d.cf == CF_SCF) {
					// Analytic-path SCF: the reference's sign coherence factor
					// applied to the real parts of the per-receiver sums.
					for (unsigned rx = 0; rx < d.numRx; ++rx) rxSumReal[rx] = rxSum[rx].real();
					f = scf<T>(rxSumReal.data(), d.numRx, d.scfP);
				} else if (d.cf == CF_MF) {
					f = mallart_fink_cf<T>(rxSum.data(), d.numRx);
				}
				std::complex<T> acc(0);
				for (unsigned rx = 0; rx < d.numRx; ++rx) acc += rxSum[rx];
				v = std::abs(acc);
			}
			value[p] = v * (T(1) / numSignals);
			factor[p] = f;
		}
	});
}

// ---------------------------------------------------------------------------
// Single-term 3D processors: one prepared A-scan per term, one term per
// signal (and per acquisition of the synthetic-y window) at each grid point.
// ---------------------------------------------------------------------------
enum SingleMode { SINGLE_T1R1_SAFT = 0, SINGLE_TNRN = 1, SINGLE_SYNTH_Y_TNRN = 2 };

template<typename T>
struct SingleDesc {
	int mode = SINGLE_T1R1_SAFT;
	unsigned numSignals = 0;     // T1R1: active elements; TnRn: numElements
	unsigned numSamples = 0;
	unsigned upsampling = 1;
	T samplingFrequency = 0;
	T propagationSpeed = 0;
	T centerFrequency = 0;
	T peakOffset = 0;
	T deadZoneM = 0;
	const T* txXY = nullptr;     // T1R1: numSignals tx positions; TnRn: [0] = first element of the group
	const T* rxXY = nullptr;     // numSignals rx positions
	const T* rxApod = nullptr;   // TnRn: numSignals weights
	T focusX = 0, focusY = 0, focusZ = 0;
	T firstTxDelay = 0;          // txDelays[0], s
	unsigned numAcq = 1;         // synthetic y: acquisitions of the window
	const T* acqY = nullptr;     // synthetic y: y of each acquisition of the window
	int cf = CF_NONE;
	T pcfGamma = 1;
	T scfP = 1;
	int nthreads = 1;
};

// Distance between two 3D points. Follows src/util/Geometry.h:67-75.
template<typename T>
T distance3d(T x0, T y0, T z0, T x1, T y1, T z1)
{
	const T dx = x1 - x0;
	const T dy = y1 - y0;
	const T dz = z1 - z0;
	return std::sqrt(dx * dx + dy * dy + dz * dz);
}

// Preparation of numAcq * numSignals A-scans (acquisition-major), as the
// STA preparation of one transmit event per signal.
// Follows src/user/processor/Vectorial3DT1R1SAFTProcessor.h:141-173,
// src/user/processor/Vectorial3DTnRnProcessor.h:173-205 and
// src/user/processor/SynthYVectorial3DTnRnProcessor.h:171-205.
template<typename T>
void prepare_single(const SingleDesc<T>& s, const T* rf, std::vector<std::complex<T>>& analytic)
{
	StaDesc<T> d;
	d.numTx = s.numAcq * s.numSignals;
	d.numRx = 1;
	d.numSamples = s.numSamples;
	d.upsampling = s.upsampling;
	d.samplingFrequency = s.samplingFrequency;
	d.propagationSpeed = s.propagationSpeed;
	d.centerFrequency = s.centerFrequency;
	d.deadZoneM = s.deadZoneM;
	d.nthreads = s.nthreads;
	prepare_signals<T>(d, rf, &analytic, nullptr);
}

// Per-point single terms, coherence factor over them, value = |sum| scaled.
// T1R1 SAFT follows src/user/processor/Vectorial3DT1R1SAFTProcessor.h:175-233,
// TnRn src/user/processor/Vectorial3DTnRnProcessor.h:207-279, synthetic y
// src/user/processor/SynthYVectorial3DTnRnProcessor.h:220-302.
// analytic: numAcq * numSignals * L.
template<typename T>
void single_term_das(const SingleDesc<T>& d, const std::complex<T>* analytic, unsigned L,
		const T* gridXYZ, std::size_t npix, T* value, T* factor)
{
	const T fsUp = d.samplingFrequency * d.upsampling;
	const T invCT = fsUp / d.propagationSpeed;
	const T signalOffset = (d.samplingFrequency * d.upsampling) * d.peakOffset / d.centerFrequency;
	const bool tnrn = d.mode != SINGLE_T1R1_SAFT;
	const bool synthY = d.mode == SINGLE_SYNTH_Y_TNRN;
	const unsigned numAcq = synthY ? d.numAcq : 1U;
	T d0 = 0, t0 = 0;
	if (tnrn) {
		d0 = d.firstTxDelay * fsUp;
		t0 = distance3d_z0<T>(d.txXY[0], d.txXY[1], d.focusX, d.focusY, d.focusZ) * invCT;
	}
	// centerAcq = (firstAcq + lastAcq) / 2, relative to the window.
	const T centerY = synthY ? d.acqY[(numAcq - 1U) / 2U] : T(0);
	const T valueFactor = static_cast<T>(1.0 / numAcq);
	T pcfFactor = 0;
	if (d.cf == CF_PCF) {
		const T sigma0 = kPi / std::sqrt(3.0);
		pcfFactor = d.pcfGamma / sigma0;
	}
	const std::size_t numTerms = static_cast<std::size_t>(numAcq) * d.numSignals;
	parallel_for(npix, d.nthreads, [&](std::size_t b, std::size_t e) {
		std::vector<std::complex<T>> terms(numTerms);
		std::vector<T> delayList(d.numSignals), realParts(numTerms), phi, phiAux;
		for (std::size_t p = b; p < e; ++p) {
			const T px = gridXYZ[3 * p], py = gridXYZ[3 * p + 1], pz = gridXYZ[3 * p + 2];
			std::fill(terms.begin(), terms.end(), std::complex<T>(0));
			for (unsigned a = 0; a < numAcq; ++a) {
				const T yOffset = synthY ? d.acqY[a] - centerY : T(0);
				const T qy = synthY ? py - yOffset : py;
				const std::complex<T>* acqSig = analytic + static_cast<std::size_t>(a) * d.numSignals * L;
				std::complex<T>* acqTerms = terms.data() + static_cast<std::size_t>(a) * d.numSignals;
				if (tnrn) {
					const T t1 = distance3d<T>(d.focusX, d.focusY, d.focusZ, px, qy, pz) * invCT;
					const T txDelay = (d.focusZ > 0) ? t1 + t0 + d0 : t1 - (t0 - d0);
					for (unsigned i = 0; i < d.numSignals; ++i) {
						delayList[i] = distance3d_z0<T>(d.rxXY[2 * i], d.rxXY[2 * i + 1], px, qy, pz) * invCT;
					}
					for (unsigned i = 0; i < d.numSignals; ++i) {
						const T delay = signalOffset + txDelay + delayList[i];
						const std::size_t idx = static_cast<std::size_t>(delay);
						const T k = delay - idx;
						if (idx + 1U < L) {
							const std::complex<T>* s = acqSig + static_cast<std::size_t>(i) * L + idx;
							acqTerms[i] = d.rxApod[i] * ((1 - k) * s[0] + k * s[1]);
						}
					}
				} else {
					for (unsigned i = 0; i < d.numSignals; ++i) {
						delayList[i] = distance3d_z0<T>(d.txXY[2 * i], d.txXY[2 * i + 1], px, py, pz) * invCT;
					}
					for (unsigned i = 0; i < d.numSignals; ++i) {
						const T rxDelay = distance3d_z0<T>(d.rxXY[2 * i], d.rxXY[2 * i + 1], px, py, pz) * invCT;
						const T delay = signalOffset + delayList[i] + rxDelay;
						const std::size_t idx = static_cast<std::size_t>(delay);
						const T k = delay - idx;
						if (idx + 1U < L) {
							const std::complex<T>* s = acqSig + static_cast<std::size_t>(i) * L + idx;
							acqTerms[i] += (1 - k) * s[0] + k * s[1];
						}
					}
				}
			}
			T f = 1;
			if (d.cf == CF_PCF) {
				f = pcf<T>(terms.data(), static_cast<unsigned>(numTerms), pcfFactor, phi, phiAux);
			} else if (d.cf == CF_SCF) {
				for (std::size_t i = 0; i < numTerms; ++i) realParts[i] = terms[i].real();
				f = scf<T>(realParts.data(), static_cast<unsigned>(numTerms), d.scfP);
			} else if (d.cf == CF_MF) {
				f = mallart_fink_cf<T>(terms.data(), static_cast<unsigned>(numTerms));
			}
			std::complex<T> acc(0);
			for (std::size_t i = 0; i < numTerms; ++i) acc += terms[i];
			T v = std::abs(acc);
			if (synthY) v = valueFactor * v;
			value[p] = v * (T(1) / d.numSignals);
			factor[p] = f;
		}
	});
}

// ---------------------------------------------------------------------------
// Two-medium imaging (linear array in medium 1 over an interface sampled as a
// list of (x, z) points, image in medium 2): refracted delays by Fermat's
// principle, then a tx x rx delay-and-sum per step of a sliding
// sub-aperture, summed as complex values.
// ---------------------------------------------------------------------------

// FermatPrinciple::calcBlockSizeForTwoStepSearch (src/util/FermatPrinciple.h:106-115);
// the maximum block size arrives as an unsigned number of wavelengths.
template<typename T>
unsigned fermat_block_size(unsigned n, T interfaceStep, T wavelength, unsigned maxBlockSizeInWavelengths)
{
	const T idealBlockSize = std::sqrt(n / 2.0) + 0.5;
	const T maxBlockSize = (wavelength * maxBlockSizeInWavelengths) / interfaceStep;
	const T blockSize = std::min(idealBlockSize, maxBlockSize);
	return std::max(2U, static_cast<unsigned>(blockSize));
}

// Travel time element (x1, z1) -> interface point -> (x2, z2), minimised in
// two steps (every blockSize-th point, then the points around the best one).
// Follows src/util/FermatPrinciple.h:117-165.
template<typename T>
void fermat_min_time_two_steps(unsigned blockSize, T c1, T c2, const T* ifXZ, unsigned n, T x1, T z1, T x2, T z2,
		T& tMin, unsigned& idxMin)
{
	const T invC1 = 1 / c1;
	const T invC2 = 1 / c2;
	auto time = [&](unsigned i) {
		const T px = ifXZ[2 * i], pz = ifXZ[2 * i + 1];
		const T dx1 = px - x1;
		const T dz1 = pz - z1;
		const T dx2 = x2 - px;
		const T dz2 = z2 - pz;
		return std::sqrt(dx1 * dx1 + dz1 * dz1) * invC1 + std::sqrt(dx2 * dx2 + dz2 * dz2) * invC2;
	};
	tMin = std::numeric_limits<T>::max();
	idxMin = std::numeric_limits<unsigned>::max();
	for (unsigned i = 0; i < n; i += blockSize) {
		const T t = time(i);
		if (t < tMin) {
			tMin = t;
			idxMin = i;
		}
	}
	const unsigned iBegin = (idxMin > (blockSize - 1)) ? idxMin - (blockSize - 1) : 0;
	const unsigned iEnd = std::min<unsigned>(idxMin + blockSize, n);
	for (unsigned i = iBegin; i < iEnd; ++i) {
		const T t = time(i);
		if (t < tMin) {
			tMin = t;
			idxMin = i;
		}
	}
}

// Interface point nearest in x, in two steps. Follows src/util/FermatPrinciple.h:210-238.
template<typename T>
void fermat_nearest_x_two_steps(unsigned blockSize, const T* ifXZ, unsigned n, T x, T& zIdxMin, unsigned& idxMin)
{
	T dxMin = std::numeric_limits<T>::max();
	idxMin = 0;
	for (unsigned i = 0; i < n; i += blockSize) {
		const T dx = std::abs(ifXZ[2 * i] - x);
		if (dx < dxMin) {
			dxMin = dx;
			idxMin = i;
		}
	}
	const unsigned iBegin = (idxMin > (blockSize - 1)) ? idxMin - (blockSize - 1) : 0;
	const unsigned iEnd = std::min<unsigned>(idxMin + blockSize, n);
	for (unsigned i = iBegin; i < iEnd; ++i) {
		const T dx = std::abs(ifXZ[2 * i] - x);
		if (dx < dxMin) {
			dxMin = dx;
			idxMin = i;
		}
	}
	zIdxMin = ifXZ[2 * idxMin + 1];
}

template<typename T>
struct TwoMediumDesc {
	unsigned numElements = 0, numElementsMux = 0;
	T pitch = 0, centerFrequency = 0, c1 = 0, c2 = 0, samplingFrequency = 0;
	unsigned numSamples = 0, upsampling = 1;
	T maxFermatBlockSize = 0, peakOffset = 0;
	unsigned signalStartOffset = 0;
	unsigned numAcq = 0, numTx = 0;       // acquisitions: numAcq x numTx x numElements x numSamples
	unsigned numSteps = 0;
	const unsigned* steps = nullptr;      // numSteps x (baseElemIdx, baseElem, firstTxElem, lastTxElem)
	unsigned numInterface = 0;
	const T* interfaceXZ = nullptr;
	const T* rxApod = nullptr;            // numElements
	int cf = CF_NONE;
	T pcfGamma = 1;
	int nthreads = 1;
};

// VectorialCombinedTwoMediumImagingProcessor<T>::process
// (src/user/processor/VectorialCombinedTwoMediumImagingProcessor.h:230-401, with
// CalculateDelays :403-484, PrepareData(WithOneTxElem) :486-570 and
// ProcessColumn(WithOneTxElem) :572-790). gridXZ: ncols x nrows (x, z), rows
// evenly spaced in z; out: ncols x nrows complex (rows above the interface 0).
template<typename T>
void two_medium_process(const TwoMediumDesc<T>& d, const T* rf, const T* gridXZ, unsigned ncols, unsigned nrows,
		std::complex<T>* out)
{
	if (d.numSteps == 0) throw std::invalid_argument("The list of step configurations is empty.");
	if (d.numInterface < 2) throw std::invalid_argument("The interface needs at least two points.");
	const unsigned U = d.upsampling;
	const unsigned L = d.numSamples * U;
	const T lambda2 = d.c2 / d.centerFrequency;
	const T signalOffset = (d.samplingFrequency * U) * (d.peakOffset / d.centerFrequency) - d.signalStartOffset * U;
	const T* ifXZ = d.interfaceXZ;
	const unsigned nIf = d.numInterface;
	auto gx = [&](unsigned col, unsigned row) { return gridXZ[2 * (static_cast<std::size_t>(col) * nrows + row)]; };
	auto gz = [&](unsigned col, unsigned row) { return gridXZ[2 * (static_cast<std::size_t>(col) * nrows + row) + 1]; };

	const T dxI = ifXZ[2] - ifXZ[0];
	const T dzI = ifXZ[3] - ifXZ[1];
	const T r = std::sqrt(dxI * dxI + dzI * dzI);
	const unsigned blockSize = fermat_block_size<T>(nIf, r, lambda2, static_cast<unsigned>(d.maxFermatBlockSize));

	// First imaged row of every column (the first one below the interface).
	std::vector<unsigned> minRow(ncols);
	const T zStep = gz(0, 1) - gz(0, 0);
	for (unsigned col = 0; col < ncols; ++col) {
		T zIdxMin;
		unsigned idxMin;
		fermat_nearest_x_two_steps<T>(blockSize, ifXZ, nIf, gx(col, 0), zIdxMin, idxMin);
		if (zIdxMin <= gz(col, 0)) {
			minRow[col] = 1;
		} else if (zIdxMin >= gz(col, nrows - 1)) {
			minRow[col] = nrows;
		} else {
			minRow[col] = static_cast<unsigned>(std::ceil((zIdxMin - gz(col, 0)) / zStep)) + 1;
		}
	}

	// Element x (ArrayGeometry::getElementX2D, src/util/ArrayGeometry.h:51-63) and
	// medium-1 paths element -> interface point, in medium-2 length units.
	const T c2ByC1 = d.c2 / d.c1;
	std::vector<T> xArray(d.numElementsMux);
	const T xCenter = ((d.numElementsMux - 1) * d.pitch) / 2 - T(0);
	for (unsigned e = 0; e < d.numElementsMux; ++e) xArray[e] = e * d.pitch - xCenter;
	std::vector<T> medium1(static_cast<std::size_t>(d.numElementsMux) * nIf);
	for (unsigned e = 0; e < d.numElementsMux; ++e) {
		for (unsigned i = 0; i < nIf; ++i) {
			const T dx = ifXZ[2 * i] - xArray[e];
			const T z = ifXZ[2 * i + 1];
			medium1[static_cast<std::size_t>(e) * nIf + i] = std::sqrt(dx * dx + z * z) * c2ByC1;
		}
	}

	// Delays in samples, (col, row, element): a Fermat search for the first
	// imaged row, then a walk along the interface from the previous row's point.
	const T fs = d.samplingFrequency * U;
	const T fsInvC2 = d.samplingFrequency * U / d.c2;
	const std::size_t mux = d.numElementsMux;
	std::vector<T> delay(static_cast<std::size_t>(ncols) * nrows * mux, T(0));
	parallel_for(ncols, d.nthreads, [&](std::size_t b, std::size_t e) {
		for (std::size_t col = b; col < e; ++col) {
			if (minRow[col] >= nrows) continue;
			for (unsigned elem = 0; elem < d.numElementsMux; ++elem) {
				unsigned last = 0;
				{
					const unsigned row = minRow[col];
					T tMin;
					unsigned idxMin;
					fermat_min_time_two_steps<T>(blockSize, d.c1, d.c2, ifXZ, nIf, xArray[elem], T(0),
							gx(static_cast<unsigned>(col), row), gz(static_cast<unsigned>(col), row), tMin, idxMin);
					delay[(col * nrows + row) * mux + elem] = tMin * fs;
					last = idxMin;
				}
				const T* m1 = &medium1[static_cast<std::size_t>(elem) * nIf];
				for (unsigned row = minRow[col] + 1; row < nrows; ++row) {
					const T px = gx(static_cast<unsigned>(col), row), pz = gz(static_cast<unsigned>(col), row);
					auto tc2 = [&](unsigned i) {
						const T dx = px - ifXZ[2 * i];
						const T dz = pz - ifXZ[2 * i + 1];
						return m1[i] + std::sqrt(dx * dx + dz * dz);
					};
					unsigned idxMin = last;
					T tC2Min = tc2(idxMin);
					for (unsigned i = idxMin + 1; i < nIf; ++i) {
						const T t = tc2(i);
						if (t >= tC2Min) break;
						tC2Min = t;
						idxMin = i;
					}
					if (idxMin == last) {
						for (int i = static_cast<int>(idxMin) - 1; i >= 0; --i) {
							const T t = tc2(static_cast<unsigned>(i));
							if (t >= tC2Min) break;
							tC2Min = t;
							idxMin = static_cast<unsigned>(i);
						}
					}
					delay[(col * nrows + row) * mux + elem] = tC2Min * fsInvC2;
					last = idxMin;
				}
			}
		}
	});

	// Signals: the STA preparation (upsampling, DC removal over the whole
	// A-scan, analytic signal) of every acquisition, (acq, tx, rx, L).
	StaDesc<T> pd;
	pd.numTx = d.numAcq * d.numTx;
	pd.numRx = d.numElements;
	pd.numSamples = d.numSamples;
	pd.upsampling = U;
	pd.samplingFrequency = d.samplingFrequency;
	pd.propagationSpeed = d.c1;
	pd.centerFrequency = d.centerFrequency;
	pd.deadZoneM = 0;
	pd.nthreads = d.nthreads;
	std::vector<std::complex<T>> sig;
	prepare_signals<T>(pd, rf, &sig, nullptr);

	T pcfFactor = 0;
	if (d.cf == CF_PCF) {
		const T sigma0 = kPi / std::sqrt(3.0);
		pcfFactor = d.pcfGamma / sigma0;
	}
	const bool oneTx = d.steps[2] == d.steps[3];
	const unsigned maxPosition = L - 2;
	const std::size_t acqStride = static_cast<std::size_t>(d.numTx) * d.numElements * L;
	parallel_for(ncols, d.nthreads, [&](std::size_t b, std::size_t e) {
		std::vector<std::complex<T>> rxSum(d.numElements);
		std::vector<T> phi, phiAux;
		for (std::size_t col = b; col < e; ++col) {
			for (unsigned row = 0; row < nrows; ++row) out[col * nrows + row] = std::complex<T>(0);
			for (unsigned row = minRow[col]; row < nrows; ++row) {
				std::complex<T> pointSum(0);
				for (unsigned si = 0; si < d.numSteps; ++si) {
					const unsigned* st = d.steps + 4 * si;
					const unsigned baseElemIdx = st[0], baseElem = st[1], firstTx = st[2], lastTx = st[3];
					const T* delays = &delay[(col * nrows + row) * mux + baseElem];
					std::fill(rxSum.begin(), rxSum.end(), std::complex<T>(0));
					for (unsigned tx = firstTx; tx <= lastTx; ++tx) {
						const T txOffset = signalOffset + delays[tx];
						// One transmit element: the signals of acquisition baseElemIdx, row 0.
						const std::complex<T>* p = sig.data() + baseElemIdx * acqStride +
								static_cast<std::size_t>(oneTx ? 0 : tx - firstTx) * d.numElements * L;
						for (unsigned rx = 0; rx < d.numElements; ++rx, p += L) {
							const T position = txOffset + delays[rx];
							if (position >= 0.0f) {
								const unsigned idx = static_cast<unsigned>(position);
								if (idx <= maxPosition) {
									const T k = position - idx;
									const std::complex<T> v0 = p[idx], v1 = p[idx + 1];
									if (oneTx) rxSum[rx] = v0 + k * (v1 - v0); else rxSum[rx] += v0 + k * (v1 - v0);
								} else if (oneTx) {
									rxSum[rx] = 0;
								}
							} else if (oneTx) {
								rxSum[rx] = 0;
							}
						}
					}
					std::complex<T> sum(0);
					for (unsigned rx = 0; rx < d.numElements; ++rx) sum += rxSum[rx] * d.rxApod[rx];
					if (d.cf == CF_PCF) {
						const T f = pcf<T>(rxSum.data(), d.numElements, pcfFactor, phi, phiAux);
						if (oneTx) pointSum += sum * f; else out[col * nrows + row] += sum * f;
					} else {
						if (oneTx) pointSum += sum; else out[col * nrows + row] += sum;
					}
				}
				if (oneTx) out[col * nrows + row] = pointSum;
			}
		}
	});
}

}  // namespace orc

#endif  // USGB_STA_ORACLE_HPP
