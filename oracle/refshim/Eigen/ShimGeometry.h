// ShimGeometry.h — AngleAxis, which the reference's transformed surfaces declare
// (Source/Core/TransformedSurface.h); written from the Rodrigues rotation formula.
// TEST INFRASTRUCTURE ONLY (see ShimDense.h); not on the simulated path.
#pragma once

#include "ShimDense.h"

namespace Eigen {

template <typename S> class AngleAxis {
public:
	using Vec = Matrix<S, 3, 1>;
	AngleAxis() = default;
	AngleAxis(S angle, const Vec &axis) : _angle(angle), _axis(axis) { }
	S angle() const { return _angle; }
	const Vec &axis() const { return _axis; }
	AngleAxis inverse() const { return AngleAxis(-_angle, _axis); }
	Matrix<S, 3, 3> toRotationMatrix() const {
		const S c = std::cos(_angle), s = std::sin(_angle), t = S(1) - c;
		const Vec &k = _axis;
		Matrix<S, 3, 3> m;
		m(0, 0) = c + t * k[0] * k[0];        m(0, 1) = t * k[0] * k[1] - s * k[2]; m(0, 2) = t * k[0] * k[2] + s * k[1];
		m(1, 0) = t * k[1] * k[0] + s * k[2]; m(1, 1) = c + t * k[1] * k[1];        m(1, 2) = t * k[1] * k[2] - s * k[0];
		m(2, 0) = t * k[2] * k[0] - s * k[1]; m(2, 1) = t * k[2] * k[1] + s * k[0]; m(2, 2) = c + t * k[2] * k[2];
		return m;
	}
	friend Vec operator*(const AngleAxis &a, const Vec &v) { return a.toRotationMatrix() * v; }
private:
	S _angle = S(0);
	Vec _axis = Vec::UnitX();
};
using AngleAxisd = AngleAxis<double>;
using AngleAxisf = AngleAxis<float>;

}  // namespace Eigen
