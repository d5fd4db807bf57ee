// Minimal stand-in for the subset of the FFTW3 API that the reference's FFT
// wrapper (src/fft/FFTW.{h,cpp}) uses: 1-D r2c, c2r and backward c2c plans in
// float and double, execute, destroy, alloc/free. FFTW is not installed here,
// so the transforms are computed with the oracle's own mixed-radix FFT
// (oracle/sta_oracle.hpp). Plans bind their arrays at creation, as FFTW does.
#pragma once
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../sta_oracle.hpp"

typedef double fftw_complex[2];
typedef float fftwf_complex[2];

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

namespace usgb_fftw_shim {

enum Kind { R2C, C2R, C2C };

template<typename T>
struct Plan {
	Kind kind;
	int n;
	int sign;
	T* rin;
	T (*cin)[2];
	T* rout;
	T (*cout)[2];
	orc::FFT<T> fft;
	std::vector<std::complex<T>> buf;

	void execute()
	{
		using C = std::complex<T>;
		buf.resize(static_cast<std::size_t>(n));
		switch (kind) {
		case R2C:
			for (int i = 0; i < n; ++i) buf[i] = C(rin[i], 0);
			fft.execute(buf.data(), buf.data(), -1);
			for (int k = 0; k <= n / 2; ++k) { cout[k][0] = buf[k].real(); cout[k][1] = buf[k].imag(); }
			break;
		case C2R:
			// Hermitian extension of bins 0..n/2.
			for (int k = 0; k <= n / 2; ++k) buf[k] = C(cin[k][0], cin[k][1]);
			for (int k = n / 2 + 1; k < n; ++k) buf[k] = std::conj(buf[n - k]);
			fft.execute(buf.data(), buf.data(), +1);
			for (int i = 0; i < n; ++i) rout[i] = buf[i].real();
			break;
		case C2C:
			for (int i = 0; i < n; ++i) buf[i] = C(cin[i][0], cin[i][1]);
			fft.execute(buf.data(), buf.data(), sign);
			for (int i = 0; i < n; ++i) { cout[i][0] = buf[i].real(); cout[i][1] = buf[i].imag(); }
			break;
		}
	}
};

template<typename T>
Plan<T>* make(Kind kind, int n, int sign, T* rin, T (*cin)[2], T* rout, T (*cout)[2])
{
	Plan<T>* p = new Plan<T>();
	p->kind = kind;
	p->n = n;
	p->sign = sign;
	p->rin = rin;
	p->cin = cin;
	p->rout = rout;
	p->cout = cout;
	p->fft.init(static_cast<unsigned>(n));
	return p;
}

}  // namespace usgb_fftw_shim

typedef usgb_fftw_shim::Plan<double>* fftw_plan;
typedef usgb_fftw_shim::Plan<float>* fftwf_plan;

inline fftw_plan fftw_plan_dft_r2c_1d(int n, double* in, fftw_complex* out, unsigned)
{ return usgb_fftw_shim::make<double>(usgb_fftw_shim::R2C, n, -1, in, nullptr, nullptr, out); }
inline fftwf_plan fftwf_plan_dft_r2c_1d(int n, float* in, fftwf_complex* out, unsigned)
{ return usgb_fftw_shim::make<float>(usgb_fftw_shim::R2C, n, -1, in, nullptr, nullptr, out); }
inline fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex* in, double* out, unsigned)
{ return usgb_fftw_shim::make<double>(usgb_fftw_shim::C2R, n, +1, nullptr, in, out, nullptr); }
inline fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex* in, float* out, unsigned)
{ return usgb_fftw_shim::make<float>(usgb_fftw_shim::C2R, n, +1, nullptr, in, out, nullptr); }
inline fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned)
{ return usgb_fftw_shim::make<double>(usgb_fftw_shim::C2C, n, sign, nullptr, in, nullptr, out); }
inline fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex* in, fftwf_complex* out, int sign, unsigned)
{ return usgb_fftw_shim::make<float>(usgb_fftw_shim::C2C, n, sign, nullptr, in, nullptr, out); }

inline void fftw_execute(fftw_plan p) { p->execute(); }
inline void fftwf_execute(fftwf_plan p) { p->execute(); }
inline void fftw_destroy_plan(fftw_plan p) { delete p; }
inline void fftwf_destroy_plan(fftwf_plan p) { delete p; }

inline double* fftw_alloc_real(std::size_t n) { return static_cast<double*>(std::calloc(n, sizeof(double))); }
inline float* fftwf_alloc_real(std::size_t n) { return static_cast<float*>(std::calloc(n, sizeof(float))); }
inline fftw_complex* fftw_alloc_complex(std::size_t n) { return static_cast<fftw_complex*>(std::calloc(n, sizeof(fftw_complex))); }
inline fftwf_complex* fftwf_alloc_complex(std::size_t n) { return static_cast<fftwf_complex*>(std::calloc(n, sizeof(fftwf_complex))); }
inline void fftw_free(void* p) { std::free(p); }
inline void fftwf_free(void* p) { std::free(p); }
