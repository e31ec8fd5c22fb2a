// GpuLevelSetLiquid.h — the drop-in for LevelSetLiquid<Dim> (Source/Core/LevelSetLiquid.h:16-191)
// behind the reference's Simulation interface (Common/Util/Simulation.h:10-34).
//
// Host C++ over the C ABI of include/garm.h: the class owns one garm_sim (the
// device state of one scene), keeps the builder-side set-up on the host
// (unionLevelSet / intersectLevelSet and the initial velocity, as
// LevelSetLiquidBuilder fills them, Source/Demo/LevelSetLiquidBuilder.cpp:27-64),
// and forwards initialize / advance / getTimeStep / saveFrame / loadFrame to the GPU.
// Frame files use the reference's .sav layout and names
// (LevelSetLiquid.cpp:425-526), so frames written by either side load in the other.
#pragma once

#include "garm.h"

#include <array>
#include <cmath>
#include <cstdint>
#include <fstream>
#include <functional>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

namespace garm::host {

// Mirror of PhysX::Simulation (Common/Util/Simulation.h:10-34).  The YAML
// description hook of the reference takes a plain stream here because the
// library carries no YAML dependency.
class Simulation {
protected:
	double _time = 0;

public:
	Simulation() = default;
	Simulation(const Simulation &) = delete;
	Simulation &operator=(const Simulation &) = delete;
	virtual ~Simulation() = default;

	void setTime(const double time) { _time = time; }
	virtual double getTimeStep(const unsigned frameRate, const double stepRate) const { return 1.0 / frameRate / stepRate; }

	virtual int dimension() const = 0;
	virtual void writeDescription(std::ostream &out) const = 0;
	virtual void writeFrame(const std::string &frameDir, const bool staticDraw) const = 0;
	virtual void saveFrame(const std::string &frameDir) const = 0;
	virtual void loadFrame(const std::string &frameDir) = 0;

	virtual void initialize() {}
	virtual void advance(const double dt) = 0;
};

// Errors: the reference prints and exits (LinearSystem.h:27-36, Simulator.cpp:95-98);
// here every failing call throws with the library's status.
class Error : public std::runtime_error {
public:
	garm_status status;
	Error(garm_status s, const std::string &what) : std::runtime_error(what + ": " + garm_status_string(s)), status(s) {}
};

inline void check(garm_status s, const char *what) {
	if (s != GARM_OK) throw Error(s, what);
}

template <int Dim>
class GpuLevelSetLiquid : public Simulation {
	static_assert(Dim == 2 || Dim == 3, "Dimension must be 2 or 3.");

public:
	using Vec = std::array<double, Dim>;
	using Sdf = std::function<double(const Vec &)>;

	// StaggeredGrid(boundaryWidth, spacing, resolution, center) (StaggeredGrid.h:27-36)
	GpuLevelSetLiquid(int boundaryWidth, double spacing, const std::array<int, Dim> &resolution, const Vec &center,
	                  const garm_config *cfg = nullptr, void *stream = nullptr) {
		_desc.dim = Dim;
		_desc.boundary_width = boundaryWidth;
		_desc.spacing = spacing;
		for (int a = 0; a < 3; a++) {
			_desc.resolution[a] = a < Dim ? resolution[a] : 1;
			_desc.center[a] = a < Dim ? center[a] : 0.0;
		}
		if (cfg) _cfg = *cfg;
		else check(garm_config_default(&_cfg), "garm_config_default");
		check(garm_sim_create(&_desc, &_cfg, stream, &_sim), "garm_sim_create");
		size_t n = 0;
		check(garm_sim_field_bytes(_sim, GARM_FIELD_LEVEL_SET, &n), "field_bytes");
		_levelSet.assign(n / 8, std::numeric_limits<double>::infinity());  // LevelSetLiquid.cpp:49
		check(garm_sim_field_bytes(_sim, GARM_FIELD_VELOCITY, &n), "field_bytes");
		_velocity.assign(n / 8, 0.0);
	}
	~GpuLevelSetLiquid() override { if (_sim) garm_sim_destroy(_sim); }

	int dimension() const override { return Dim; }

	// LevelSetLiquid::getTimeStep (LevelSetLiquid.h:129): stepRate * dx / max|u|
	double getTimeStep(const unsigned frameRate, const double stepRate) const override {
		(void)frameRate;
		double dt = 0;
		check(garm_sim_time_step(_sim, stepRate, &dt), "garm_sim_time_step");
		return dt;
	}

	// Builder-side set-up (LevelSetLiquid.cpp:700-716), evaluated at cell centres.
	void unionLevelSet(const Sdf &sdf) { forEachCell([&](size_t i, const Vec &p) { _levelSet[i] = std::min(_levelSet[i], sdf(p)); }); }
	void intersectLevelSet(const Sdf &sdf) { forEachCell([&](size_t i, const Vec &p) { _levelSet[i] = std::max(_levelSet[i], sdf(p)); }); }
	// The staggered velocity in .sav order (D face arrays); callers may fill it before initialize().
	std::vector<double> &initialVelocity() { return _velocity; }
	void setUniformVelocity(int axis, double v) {
		size_t off = 0;
		for (int a = 0; a < Dim; a++) {
			size_t cnt = 1;
			for (int b = 0; b < Dim; b++) cnt *= size_t(_desc.resolution[b] + (a == b ? 1 : 0));
			for (size_t i = 0; i < cnt; i++) _velocity[off + i] = (a == axis) ? v : _velocity[off + i];
			off += cnt;
		}
	}

	// LevelSetLiquid::initialize (LevelSetLiquid.cpp:528-598)
	void initialize() override {
		check(garm_sim_upload(_sim, GARM_FIELD_LEVEL_SET, _levelSet.data(), _levelSet.size() * 8), "upload levelSet");
		check(garm_sim_upload(_sim, GARM_FIELD_VELOCITY, _velocity.data(), _velocity.size() * 8), "upload velocity");
		const garm_status s = garm_sim_initialize(_sim);
		if (s != GARM_OK && s != GARM_NOT_CONVERGED) throw Error(s, "garm_sim_initialize");
	}

	// LevelSetLiquid::restart (LevelSetLiquid.cpp:1285-1352)
	void restart() { check(garm_stage_restart(_sim), "garm_stage_restart"); }

	// LevelSetLiquid::advance (LevelSetLiquid.cpp:608-698)
	void advance(const double dt) override {
		const garm_status s = garm_sim_advance(_sim, dt, &_lastStats);
		if (s != GARM_OK && s != GARM_NOT_CONVERGED) throw Error(s, "garm_sim_advance");
		_restarted.push_back(_lastStats.restarted);
	}

	void writeDescription(std::ostream &out) const override {
		out << "dimension: " << Dim << "\nobjects:\n  - name: liquid\n    data_mode: dynamic\n";
	}

	// Frame output: the rendered level set (_tmpLevelSet) as raw doubles.  Meshing
	// (Contourer / SurfaceMesh) stays outside the GPU step and outside this library.
	void writeFrame(const std::string &frameDir, const bool) const override {
		writeField(frameDir + "/levelSet.bin", GARM_FIELD_TMP_LEVEL_SET);
	}

	// LevelSetLiquid::saveFrame (LevelSetLiquid.cpp:425-471), RM+GA; ψ0 too in the Newton configuration
	void saveFrame(const std::string &frameDir) const override {
		writeField(frameDir + "/velocity.sav", GARM_FIELD_VELOCITY);
		writeField(frameDir + "/refMap.sav", GARM_FIELD_REF_MAP);
		writeField(frameDir + "/refLevelSet.sav", GARM_FIELD_REF_LEVEL_SET);
		writeField(frameDir + "/advRegion.sav", GARM_FIELD_ADV_REGION);
		writeField(frameDir + "/refMapGrad.sav", GARM_FIELD_REF_MAP_GRAD);
		if (_cfg.restart_newton) writeField(frameDir + "/refLevelSetGrad.sav", GARM_FIELD_REF_LEVEL_SET_GRAD);
	}

	// LevelSetLiquid::loadFrame (LevelSetLiquid.cpp:474-526)
	void loadFrame(const std::string &frameDir) override {
		readField(frameDir + "/velocity.sav", GARM_FIELD_VELOCITY);
		readField(frameDir + "/refMap.sav", GARM_FIELD_REF_MAP);
		readField(frameDir + "/refLevelSet.sav", GARM_FIELD_REF_LEVEL_SET);
		readField(frameDir + "/advRegion.sav", GARM_FIELD_ADV_REGION);
		readField(frameDir + "/refMapGrad.sav", GARM_FIELD_REF_MAP_GRAD);
		if (_cfg.restart_newton) readField(frameDir + "/refLevelSetGrad.sav", GARM_FIELD_REF_LEVEL_SET_GRAD);
		check(garm_sim_finish_load(_sim), "garm_sim_finish_load");
	}

	const garm_step_stats &lastStats() const { return _lastStats; }
	const std::vector<int> &restarted() const { return _restarted; }
	garm_sim *handle() const { return _sim; }
	const garm_grid_desc &desc() const { return _desc; }

	std::vector<double> download(int field) const {
		size_t n = 0;
		check(garm_sim_field_bytes(_sim, field, &n), "field_bytes");
		std::vector<double> v(n / 8);
		check(garm_sim_download(_sim, field, v.data(), n), "download");
		return v;
	}

private:
	garm_grid_desc _desc{};
	garm_config _cfg{};
	garm_sim *_sim = nullptr;
	std::vector<double> _levelSet, _velocity;
	garm_step_stats _lastStats{};
	std::vector<int> _restarted;

	template <typename F>
	void forEachCell(F &&f) {
		const double dx = _desc.spacing;
		double cellOrigin[3];
		for (int a = 0; a < Dim; a++) cellOrigin[a] = (_desc.center[a] - double(_desc.resolution[a]) * dx / 2) + 1.0 * dx / 2;
		const int nz = Dim == 3 ? _desc.resolution[2] : 1;
		size_t i = 0;
		for (int k = 0; k < nz; k++)
			for (int j = 0; j < _desc.resolution[1]; j++)
				for (int c = 0; c < _desc.resolution[0]; c++, i++) {
					Vec p;
					p[0] = cellOrigin[0] + double(c) * dx;
					p[1] = cellOrigin[1] + double(j) * dx;
					if constexpr (Dim == 3) p[2] = cellOrigin[2] + double(k) * dx;
					f(i, p);
				}
	}

	void writeField(const std::string &path, int field) const {
		size_t n = 0;
		check(garm_sim_field_bytes(_sim, field, &n), "field_bytes");
		std::vector<char> buf(n);
		check(garm_sim_download(_sim, field, buf.data(), n), "download");
		std::ofstream out(path, std::ios::binary);
		if (!out) throw Error(GARM_INVALID, "cannot open " + path);
		out.write(buf.data(), std::streamsize(n));
	}

	void readField(const std::string &path, int field) {
		size_t n = 0;
		check(garm_sim_field_bytes(_sim, field, &n), "field_bytes");
		std::vector<char> buf(n);
		std::ifstream in(path, std::ios::binary);
		if (!in || !in.read(buf.data(), std::streamsize(n))) throw Error(GARM_INVALID, "cannot read " + path);
		check(garm_sim_upload(_sim, field, buf.data(), n), "upload");
	}
};

// Simulator::advanceTimeBySteps (Common/Util/Simulator.cpp:102-128): frame-clamped
// steps of stepRate * dx / max|u|.  Returns the number of steps taken.
inline int advanceTimeBySteps(Simulation &sim, unsigned frameRate, double stepRate, double targetTime) {
	double time = 0;
	bool done = time >= targetTime;
	int steps = 0;
	while (!done) {
		double dt = sim.getTimeStep(frameRate, stepRate);
		if (time + dt >= targetTime) {
			dt = targetTime - time;
			done = true;
		} else if (time + 2 * dt >= targetTime)
			dt = (targetTime - time) / 2;
		sim.advance(dt);
		time += dt;
		steps++;
	}
	return steps;
}

}  // namespace garm::host
