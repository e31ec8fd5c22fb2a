// garm_demo.cpp — the reference demo's flow (Source/Demo/Demo.cpp:24-56,
// Common/Util/Simulator.cpp:13-70) through GpuLevelSetLiquid: build a dam-break
// scene on the host, initialize, run frames with the Simulator dt policy, save a
// frame, load it into a second instance and check that both continue identically.
//
//   garm_demo <dim> <n> <frames> <outdir>
#include "GpuLevelSetLiquid.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <memory>

using namespace garm::host;

template <int Dim>
static int run(int n, int frames, const std::string &out) {
	using L = GpuLevelSetLiquid<Dim>;
	typename L::Vec center;
	std::array<int, Dim> res;
	for (int a = 0; a < Dim; a++) { center[a] = 0.5; res[a] = n + 4; }
	auto makeLiquid = [&]() {
		auto liquid = std::make_unique<L>(2, 1.0 / n, res, center);
		// ImplicitBox over [-1, e]: the liquid column {x < .4, y < .5(.6), z < .6}
		const double e[3] = {0.4, Dim == 2 ? 0.6 : 0.5, 0.6};
		liquid->unionLevelSet([&](const typename L::Vec &p) {
			double phi[Dim], mx = -1e300, s = 0;
			bool inside = true;
			for (int a = 0; a < Dim; a++) {
				const double lo = -1.0, len = e[a] - lo, c = lo + len / 2, h = len / 2;
				phi[a] = std::abs(p[a] - c) - h;
				inside = inside && phi[a] <= 0;
				mx = std::max(mx, phi[a]);
				const double q = std::max(phi[a], 0.0);
				s += q * q;
			}
			return inside ? mx : std::sqrt(s);
		});
		return liquid;
	};
	auto liquid = makeLiquid();
	liquid->initialize();
	liquid->restart();
	int steps = 0;
	for (int f = 1; f <= frames; f++) {
		liquid->setTime((f - 1.0) / 25);
		steps += advanceTimeBySteps(*liquid, 25, 1.0, 1.0 / 25);
		const auto &st = liquid->lastStats();
		std::printf("frame %d: steps %d, cg %d it, %d unknowns, residual %.2e, restarted %d, %.2f ms\n", f, steps, st.cg_iterations,
		            st.unknowns, st.cg_residual, st.restarted, st.ms_total);
	}
	std::filesystem::create_directories(out);
	liquid->saveFrame(out);
	liquid->writeFrame(out, false);

	auto resumed = makeLiquid();
	resumed->loadFrame(out);
	liquid->advance(0.01);
	resumed->advance(0.01);
	const auto a = liquid->download(GARM_FIELD_LEVEL_SET), b = resumed->download(GARM_FIELD_LEVEL_SET);
	double diff = 0;
	for (size_t i = 0; i < a.size(); i++) diff = std::max(diff, std::abs(a[i] - b[i]));
	std::printf("resume check: max |phi - phi_resumed| = %.3e\n", diff);
	return diff <= 1e-12 ? 0 : 2;
}

int main(int argc, char **argv) {
	const int dim = argc > 1 ? std::atoi(argv[1]) : 3;
	const int n = argc > 2 ? std::atoi(argv[2]) : 32;
	const int frames = argc > 3 ? std::atoi(argv[3]) : 2;
	const std::string out = argc > 4 ? argv[4] : "garm_demo_out";
	try {
		return dim == 2 ? run<2>(n, frames, out) : run<3>(n, frames, out);
	} catch (const std::exception &e) {
		std::fprintf(stderr, "garm_demo: %s\n", e.what());
		return 1;
	}
}
