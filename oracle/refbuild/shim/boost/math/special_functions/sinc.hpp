// Minimal stand-in for boost::math::sinc_pi: sin(x)/x, with the Taylor series
// 1 - x^2/6 + x^4/120 for |x| below eps^(1/4) (Boost's published method).
#pragma once
#include <cmath>
#include <limits>
namespace boost { namespace math {
template<typename T>
T sinc_pi(T x)
{
	const T eps = std::numeric_limits<T>::epsilon();
	const T b0 = eps, b2 = std::sqrt(eps), bn = std::sqrt(b2);
	const T ax = std::abs(x);
	if (ax >= bn) return std::sin(x) / x;
	T r = 1;
	if (ax >= b0) {
		const T x2 = x * x;
		r -= x2 / 6;
		if (ax >= b2) r += x2 * x2 / 120;
	}
	return r;
}
}}  // namespace boost::math
