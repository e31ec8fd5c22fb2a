// gcc_compat.h — force-included (g++ -include) ahead of every reference source compiled
// into oracle/_ref.  TEST INFRASTRUCTURE ONLY.
//
// The reference deduces an `int` template parameter from the extent of a std::array,
// whose type is std::size_t: the loops over the D face grids (Source/Core/Grid.h:106-121)
// and Reinitialization::advance's stencil length (Source/Core/Reinitialization.h:20-21).
// The standard makes such a deduction fail ([temp.deduct.type]: the type of the argument
// must match the type of the template parameter) and g++ follows it, so the unmodified
// sources do not compile with g++ as shipped.  This header adds overloads that g++ can
// deduce and that do exactly what the reference's do: the array loops visit the grids in
// axis order with the same per-grid loop.
//
// Reinitialization::advance has a second construct g++ rejects: it calls the member
// template GridBasedData::stencil of a dependent object without the `template` keyword
// (Reinitialization.h:31), which g++ parses as a comparison.  So advance is restated here,
// statement for statement, for the three stencil lengths the reference uses (3, 5, 7);
// the reference's template is then never instantiated.  Everything it calls (the WENO5
// and ENO derivatives, GridBasedData::stencil, parallelForEach) is the reference's own.
#pragma once

#include "Grid.h"
#include "GridBasedData.h"

#include <array>
#include <cstddef>
#include <functional>
#include <utility>

namespace PhysX {

template <int Dim, std::size_t N, typename Func>
	requires (N == std::size_t(Dim)) && std::is_convertible_v<Func, std::function<void(const int, const Vector<Dim, int> &)>>
inline void forEach(const std::array<Grid<Dim>, N> &grids, const Func func)
{
	for (int axis = 0; axis < Dim; axis++)
		forEach(grids[axis], std::bind(func, axis, std::placeholders::_1));
}

template <int Dim, std::size_t N, typename Func>
	requires (N == std::size_t(Dim)) && std::is_convertible_v<Func, std::function<void(const int, const Vector<Dim, int> &)>>
inline void parallelForEach(const std::array<Grid<Dim>, N> &grids, const Func func)
{
	for (int axis = 0; axis < Dim; axis++)
		parallelForEach<Dim>(grids[axis], std::bind(func, axis, std::placeholders::_1));
}

namespace Reinitialization {

// Reinitialization.h:20-48: one forward-Euler step of φ_τ = sgn(φ)(1 - |∇φ|) with the
// Godunov upwind combination of the one-sided derivatives, the smoothed sign
// φ / sqrt(φ² + (dx |∇φ|)²), and the reference's order of operations.
#define GARM_REF_ADVANCE_LEN(L)                                                                                     \
	template <int Dim>                                                                                              \
	inline void advance(const GridBasedData<Dim, double> &field, GridBasedData<Dim, double> &newField, const double dt, \
	                    std::pair<double, double> (*getDrv)(const std::array<double, L> &, const double))           \
	{                                                                                                               \
		DECLARE_DIM_TYPES(Dim)                                                                                      \
		const auto square = [](const double x) { return x * x; };                                                   \
		const auto sign = [](const double val, const double sp) { return val / std::sqrt(val * val + sp * sp); };  \
		parallelForEach(field.grid, [&](const VectorDi &coord) {                                                    \
			std::pair<double, double> drv[Dim];                                                                     \
			for (int axis = 0; axis < Dim; axis++)                                                                  \
				drv[axis] = getDrv(field.template stencil<L - 1>(coord - VectorDi::Unit(axis) * (L >> 1), axis),    \
				                   field.grid.invSpacing);                                                          \
			double sum = 0;                                                                                         \
			if (field[coord] < 0) {                                                                                 \
				for (int axis = 0; axis < Dim; axis++) {                                                            \
					sum += square(std::min(drv[axis].first, 0.0));                                                  \
					sum += square(std::max(drv[axis].second, 0.0));                                                \
				}                                                                                                   \
			}                                                                                                       \
			else {                                                                                                  \
				for (int axis = 0; axis < Dim; axis++) {                                                            \
					sum += square(std::max(drv[axis].first, 0.0));                                                  \
					sum += square(std::min(drv[axis].second, 0.0));                                                 \
				}                                                                                                   \
			}                                                                                                       \
			sum = std::sqrt(sum);                                                                                   \
			newField[coord] = field[coord] + dt * sign(field[coord], field.grid.spacing * sum) * (1 - sum);         \
		});                                                                                                         \
	}
GARM_REF_ADVANCE_LEN(3)
GARM_REF_ADVANCE_LEN(5)
GARM_REF_ADVANCE_LEN(7)
#undef GARM_REF_ADVANCE_LEN

}  // namespace Reinitialization

}  // namespace PhysX
