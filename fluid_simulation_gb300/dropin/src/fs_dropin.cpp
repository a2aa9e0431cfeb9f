// Implementation of the drop-in classes over the fsgpu C ABI.  Every
// simulation phase runs on the GPU; the host objects are mirrors that are
// downloaded lazily after GPU work and uploaded before the next GPU work
// when the caller changed them.  The reference behaviour each method keeps
// is cited at the method.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <utility>

#include "fsgpu.h"

#include <FluidDomain.h>
#include <FluidSolver.h>
#include <LevelSet.h>
#include <MacGrid.h>
#include <MarkerParticleSet.h>

namespace {

void check(fs_handle* h, int rc)
{
    if (rc != FS_OK) throw std::runtime_error(fs_last_error(h));
}

const int kGridId[8] = {FS_U_FRONT, FS_V_FRONT, FS_U_BACK, FS_V_BACK, FS_U_PREV, FS_V_PREV, FS_U_DIFF, FS_V_DIFF};

const char* kValidateMessage =
    "Memory pool and fluid domain does not match. Initialize the fluid solver with a memory pool corresponding "
    "to the right fluid domain!";

}  // namespace

// ---------------------------------------------------------------- MacGrid

MacGrid::MacGrid(int size_x, int size_y, MyFloat length_x, MyFloat length_y)
    : GridInterface(size_x, size_y, length_x / size_x, length_y / size_y), _h(nullptr),
      _cell_type_buffer(size_x, size_y)
{
    for (int b = 0; b < NBUF; ++b) _buf[b] = new Grid<MyFloat>(size_x, size_y, _DELTA_X, _DELTA_Y);
    for (int b = 0; b <= NBUF; ++b) _stale[b] = _dirty[b] = false;
    clearCellTypeBuffer();  // src/MacGrid.cpp:24
    _dirty[NBUF] = false;   // a new device grid starts with the same cell types
}

MacGrid::~MacGrid()
{
    for (int b = 0; b < NBUF; ++b) delete _buf[b];
}

void MacGrid::attach(fs_handle* h) { _h = h; }

void MacGrid::pull(int b) const
{
    if (b == NBUF) {
        std::vector<uint8_t> lab(static_cast<size_t>(_SIZE_X) * _SIZE_Y);
        check(_h, fs_get_labels(_h, lab.data()));
        CellType* out = _cell_type_buffer.raw();
        for (size_t c = 0; c < lab.size(); ++c) out[c] = static_cast<CellType>(lab[c]);
    } else {
        check(_h, fs_get_grid(_h, kGridId[b], _buf[b]->raw()));
    }
    _stale[b] = false;
}

const Grid<MyFloat>& MacGrid::rd(Buf b) const
{
    if (_stale[b]) pull(b);
    return *_buf[b];
}

Grid<MyFloat>& MacGrid::wr(Buf b)
{
    if (_stale[b]) pull(b);
    _dirty[b] = true;
    return *_buf[b];
}

const Grid<CellType>& MacGrid::labels() const
{
    if (_stale[NBUF]) pull(NBUF);
    return _cell_type_buffer;
}

Grid<CellType>& MacGrid::labelsW()
{
    if (_stale[NBUF]) pull(NBUF);
    _dirty[NBUF] = true;
    return _cell_type_buffer;
}

void MacGrid::push()
{
    if (!_h) return;
    for (int b = 0; b < NBUF; ++b)
        if (_dirty[b]) {
            check(_h, fs_set_grid(_h, kGridId[b], _buf[b]->raw()));
            _dirty[b] = false;
        }
    if (_dirty[NBUF]) {
        const CellType* in = _cell_type_buffer.raw();
        std::vector<uint8_t> lab(static_cast<size_t>(_SIZE_X) * _SIZE_Y);
        for (size_t c = 0; c < lab.size(); ++c) lab[c] = static_cast<uint8_t>(in[c]);
        check(_h, fs_set_labels(_h, lab.data()));
        _dirty[NBUF] = false;
    }
}

void MacGrid::invalidate()
{
    if (!_h) return;
    for (int b = 0; b <= NBUF; ++b) _stale[b] = true;
}

// src/MacGrid.cpp:32-50: border SOLID, interior AIR.
void MacGrid::clearCellTypeBuffer()
{
    Grid<CellType>& g = labelsW();
    for (int j = 0; j < _SIZE_Y; ++j)
        for (int i = 0; i < _SIZE_X; ++i)
            g(i, j) = (i > 0 && j > 0 && i < _SIZE_X - 1 && j < _SIZE_Y - 1) ? AIR : SOLID;
}

// src/MacGrid.cpp:52-56.
void MacGrid::updatePreviousVelocityBuffer()
{
    if (_h) {
        push();
        check(_h, fs_phase(_h, FS_PH_SAVE_PREV, 0.0f));
        _stale[UP] = _stale[VP] = true;
        return;
    }
    *_buf[UP] = *_buf[UF];
    *_buf[VP] = *_buf[VF];
}

// src/MacGrid.cpp:58-70.
void MacGrid::updateVelocityDiffBuffer()
{
    if (_h) {
        push();
        check(_h, fs_phase(_h, FS_PH_SAVE_DIFF, 0.0f));
        _stale[UD] = _stale[VD] = true;
        return;
    }
    for (int j = 0; j < _SIZE_Y; ++j)
        for (int i = 0; i < _SIZE_X; ++i) {
            (*_buf[UD])(i, j) = _buf[UF]->value(i, j) - _buf[UP]->value(i, j);
            (*_buf[VD])(i, j) = _buf[VF]->value(i, j) - _buf[VP]->value(i, j);
        }
}

// src/MacGrid.cpp:89-93.
void MacGrid::swapVelocityBuffers()
{
    if (_h) {
        push();
        check(_h, fs_phase(_h, FS_PH_SWAP, 0.0f));
    }
    std::swap(_buf[UF], _buf[UB]);
    std::swap(_buf[VF], _buf[VB]);
    std::swap(_stale[UF], _stale[UB]);
    std::swap(_stale[VF], _stale[VB]);
}

// ---------------------------------------------------------------- MarkerParticleSet

MarkerParticleSet::MarkerParticleSet(int size)
    : _h(nullptr), _particles(static_cast<size_t>(size)), _stale(false), _modified(size > 0), _synced(0)
{
}

MarkerParticleSet::~MarkerParticleSet() {}

void MarkerParticleSet::attach(fs_handle* h)
{
    _h = h;
    _modified = true;
}

// Downloads the particles the device holds (the first _synced ones; particles
// appended since then are not on the device yet and stay as they are).
void MarkerParticleSet::pull() const
{
    if (!_stale || !_h) return;
    if (_synced > 0)
        check(_h, fs_get_particles(_h, reinterpret_cast<float*>(_particles.data()), static_cast<int64_t>(_synced)));
    _stale = false;
}

void MarkerParticleSet::push()
{
    if (!_h) return;
    if (_modified) {
        check(_h, fs_set_particles(_h, reinterpret_cast<const float*>(_particles.data()),
                                   static_cast<int64_t>(_particles.size())));
    } else if (_synced < _particles.size()) {
        check(_h, fs_add_particles(_h, reinterpret_cast<const float*>(_particles.data() + _synced),
                                   static_cast<int64_t>(_particles.size() - _synced)));
    }
    _modified = false;
    _synced = _particles.size();
}

void MarkerParticleSet::invalidate()
{
    if (_h) _stale = true;
}

// The next host access downloads all n: the device holds every particle.
void MarkerParticleSet::deviceAppended(std::size_t n)
{
    _particles.resize(n);
    _synced = n;
    _stale = true;
}

// Appends without downloading: the device keeps its newer copy of the
// particles before this one, and only the appended ones are uploaded.
void MarkerParticleSet::addParticle(MarkerParticle p) { _particles.push_back(p); }

void MarkerParticleSet::reserve(int particle_count) { _particles.reserve(static_cast<size_t>(particle_count)); }

void MarkerParticleSet::clear()
{
    _particles.clear();
    _stale = false;
    _modified = true;
}

int MarkerParticleSet::size() const { return static_cast<int>(_particles.size()); }

MarkerParticleSet::iterator MarkerParticleSet::begin()
{
    pull();
    _modified = true;
    return _particles.begin();
}

MarkerParticleSet::iterator MarkerParticleSet::end()
{
    pull();
    _modified = true;
    return _particles.end();
}

MarkerParticleSet::const_iterator MarkerParticleSet::begin() const
{
    pull();
    return _particles.cbegin();
}

MarkerParticleSet::const_iterator MarkerParticleSet::end() const
{
    pull();
    return _particles.cend();
}

// src/MarkerParticleSet.cpp:40-46.
void MarkerParticleSet::advect(MyFloat dt)
{
    if (_h) {
        push();
        check(_h, fs_phase(_h, FS_PH_ADVECT, dt));
        invalidate();
        return;
    }
    for (auto& p : _particles) p.advect(dt);
}

// src/MarkerParticleSet.cpp:48-62, against the cell types of the domain's grid.
void MarkerParticleSet::advectAndEnsureOutsideObstacles(MyFloat dt, const MacGrid& mac_grid)
{
    if (_h) {
        const_cast<MacGrid&>(mac_grid).push();
        push();
        check(_h, fs_phase(_h, FS_PH_ADVECT_SAFE, dt));
        invalidate();
        return;
    }
    for (auto& p : _particles) {
        p.advect(dt);
        const int x = p.posX() / mac_grid.deltaX();
        const int y = p.posY() / mac_grid.deltaY();
        if (mac_grid.cellType(x, y) == SOLID) p.advect(-dt);
    }
}

// ---------------------------------------------------------------- LevelSet (host only)

LevelSet::LevelSet(int size_x, int size_y, MyFloat length_x, MyFloat length_y)
    : Grid<MyFloat>(size_x, size_y, length_x / size_x, length_y / size_y)
{
}

MyFloat LevelSet::distance(int from_i, int from_j, int to_i, int to_j)
{
    const MyFloat di = to_i - from_i, dj = to_j - from_j;
    return std::sqrt(di * di + dj * dj);
}

// src/LevelSet.cpp:27-42: one-sided difference against the velocity sign.
MyFloat LevelSet::computeUpwindGradientX(int i, int j, MyFloat vel_x)
{
    const int ip = CLAMP(i + 1, 0, _SIZE_X - 1), im = CLAMP(i - 1, 0, _SIZE_X - 1);
    i = CLAMP(i, 0, _SIZE_X - 1);
    j = CLAMP(j, 0, _SIZE_Y - 1);
    return vel_x < 0 ? (*this)(ip, j) - (*this)(i, j) : (*this)(i, j) - (*this)(im, j);
}

MyFloat LevelSet::computeUpwindGradientY(int i, int j, MyFloat vel_y)
{
    const int jp = CLAMP(j + 1, 0, _SIZE_Y - 1), jm = CLAMP(j - 1, 0, _SIZE_Y - 1);
    i = CLAMP(i, 0, _SIZE_X - 1);
    j = CLAMP(j, 0, _SIZE_Y - 1);
    return vel_y < 0 ? (*this)(i, jp) - (*this)(i, j) : (*this)(i, j) - (*this)(i, jm);
}

// ---------------------------------------------------------------- FluidSource / FluidDomain

FluidSource::FluidSource(BBox<MyFloat> area, MyFloat delta_x, MyFloat delta_y, MyFloat x_velocity,
                         MyFloat y_velocity, MyFloat time_step, int max_spawns)
    : _area(area), _x_velocity(x_velocity), _y_velocity(y_velocity), _delta_x(delta_x), _delta_y(delta_y),
      _time_step(time_step), _time_since_last(0.0), _max_spawns(max_spawns), _n_spawns(0)
{
}

FluidSource::~FluidSource() {}

// src/FluidDomain.cpp:29-52: a lattice of spacing delta / 2.5 over the area,
// every time_step, at most max_spawns times (-1: unlimited).
void FluidSource::update(MarkerParticleSet& particle_set, MyFloat dt)
{
    if (isFinished()) return;
    if (_time_since_last >= _time_step) {
        const MyFloat x_incr = _delta_x / 2.5;
        const MyFloat y_incr = _delta_y / 2.5;
        for (MyFloat y = _area.y_min; y < _area.y_max; y += y_incr)
            for (MyFloat x = _area.x_min; x < _area.x_max; x += x_incr)
                particle_set.addParticle(MarkerParticle(x, y, _x_velocity, _y_velocity));
        _time_since_last = 0;
        _n_spawns++;
    }
    _time_since_last += dt;
}

FluidDomain::FluidDomain(int size_x, int size_y, MyFloat length_x, MyFloat length_y, MyFloat density,
                         MyFloat pic_ratio)
    : GridInterface(size_x, size_y, length_x / size_x, length_y / size_y), _h(nullptr), _density(density),
      _pic_ratio(pic_ratio), _mac_grid(size_x, size_y, length_x, length_y),
      _level_set(size_x, size_y, length_x, length_y)
{
    fs_config c;
    fs_config_init(&c, size_x, size_y);
    c.length_x = length_x;
    c.length_y = length_y;
    c.density = density;
    c.pic_ratio = pic_ratio;
    if (fs_create(&c, &_h) != FS_OK) throw std::runtime_error(fs_last_error(nullptr));
    _mac_grid.attach(_h);
    _particle_set.attach(_h);
}

FluidDomain::~FluidDomain() { fs_destroy(_h); }

// src/FluidDomain.cpp:75-78; the source (with its timing state) lives on the
// device, which spawns its particles there.
void FluidDomain::addFluidSource(FluidSource s)
{
    const BBox<MyFloat>& a = s._area;
    check(_h, fs_add_fluid_source(_h, a.x_min, a.x_max, a.y_min, a.y_max, s._delta_x, s._delta_y, s._x_velocity,
                                  s._y_velocity, s._time_step, s._max_spawns));
    int n = 0;
    check(_h, fs_num_fluid_sources(_h, &n));
    check(_h, fs_set_fluid_source_state(_h, n - 1, s._time_since_last, s._n_spawns));
    _fluid_sources.push_back(s);
}

// src/FluidDomain.cpp:80-87: every source's FluidSource::update, on the device.
void FluidDomain::update(MyFloat dt)
{
    _particle_set.push();  // host additions first, as they came first
    int64_t before = 0, after = 0;
    check(_h, fs_num_particles(_h, &before));
    check(_h, fs_update(_h, dt));
    check(_h, fs_num_particles(_h, &after));
    if (after != before) _particle_set.deviceAppended(static_cast<std::size_t>(after));
}

void FluidDomain::clearFluidSources()
{
    check(_h, fs_clear_fluid_sources(_h));
    _fluid_sources.clear();
}
void FluidDomain::resetParticleSet() { _particle_set.clear(); }

// src/FluidDomain.cpp:99-102.
void FluidDomain::setPicRatio(MyFloat pic_ratio)
{
    _pic_ratio = CLAMP(pic_ratio, 0, 1);
    check(_h, fs_set_pic_ratio(_h, pic_ratio));
}

MacGrid& FluidDomain::macGrid() { return _mac_grid; }
LevelSet& FluidDomain::levelSet() { return _level_set; }
MarkerParticleSet& FluidDomain::markerParticleSet() { return _particle_set; }
const MacGrid& FluidDomain::macGrid() const { return _mac_grid; }
const LevelSet& FluidDomain::levelSet() const { return _level_set; }
const MarkerParticleSet& FluidDomain::markerParticleSet() const { return _particle_set; }
const MyFloat FluidDomain::density() const { return _density; }
const MyFloat FluidDomain::picRatio() const { return _pic_ratio; }

void FluidDomain::pushToDevice()
{
    _mac_grid.push();
    _particle_set.push();
}

void FluidDomain::deviceUpdated()
{
    _mac_grid.invalidate();
    _particle_set.invalidate();
}

// src/FluidDomain.cpp:150-180 (on the GPU); it labels from the domain's own
// particle set, whatever set is passed, as the reference does.
void FluidDomain::classifyCells(MarkerParticleSet&)
{
    pushToDevice();
    check(_h, fs_phase(_h, FS_PH_CLASSIFY, 0.0f));
    deviceUpdated();
}

// src/FluidDomain.cpp:127-148 on the GPU; like the reference it labels from
// the domain's own level set, whatever level set is passed.
void FluidDomain::classifyCells(LevelSet&)
{
    pushToDevice();
    check(_h, fs_set_level_set(_h, _level_set.raw()));
    check(_h, fs_classify_level_set(_h));
    deviceUpdated();
}

// src/FluidDomain.cpp:104-125 on the GPU (the level set goes to the device,
// is advected there with the device's velocities, and comes back).
void FluidDomain::advectLevelSet(MyFloat dt)
{
    pushToDevice();
    check(_h, fs_set_level_set(_h, _level_set.raw()));
    check(_h, fs_advect_level_set(_h, dt));
    check(_h, fs_get_level_set(_h, _level_set.raw()));
}

// ---------------------------------------------------------------- FluidSolverMemoryPool / FluidSolver

FluidSolverMemoryPool::FluidSolverMemoryPool(int size_x, int size_y, MyFloat delta_x, MyFloat delta_y)
    : GridInterface(size_x, size_y, delta_x, delta_y)
{
}

FluidSolverMemoryPool::FluidSolverMemoryPool(const FluidDomain& d)
    : GridInterface(d.sizeX(), d.sizeY(), d.deltaX(), d.deltaY())
{
}

// As src/FluidSolver.cpp:56-62: the copy keeps delta_x for both deltas.
FluidSolverMemoryPool::FluidSolverMemoryPool(const FluidSolverMemoryPool& other)
    : GridInterface(other.sizeX(), other.sizeY(), other.deltaX(), other.deltaX())
{
}

FluidSolverMemoryPool::~FluidSolverMemoryPool() {}

// src/FluidSolver.cpp:78-82: at most 100 CG updates, Eigen's default tolerance.
FluidSolver::FluidSolver(FluidSolverMemoryPool mem_pool)
    : _mem_pool(mem_pool), _cg_max_iterations(100),
      _cg_tolerance(std::numeric_limits<MyFloat>::epsilon())
{
}

FluidSolver::~FluidSolver() {}

// src/FluidSolver.cpp:89-97.
bool FluidSolver::validate(const FluidDomain& d)
{
    return d.sizeX() == _mem_pool.sizeX() && d.sizeY() == _mem_pool.sizeY() &&
           std::abs(d.deltaX() - _mem_pool.deltaX()) < 0.0000001 &&
           std::abs(d.deltaY() - _mem_pool.deltaY()) < 0.0000001;
}

void FluidSolver::step(FluidDomain& d, int method, MyFloat dt)
{
    if (!validate(d)) throw std::runtime_error(kValidateMessage);
    d.pushToDevice();
    check(d.handle(), fs_set_cg(d.handle(), _cg_tolerance, _cg_max_iterations));
    check(d.handle(), fs_step(d.handle(), method, dt));
    d.deviceUpdated();
}

void FluidSolver::stepSemiLagrangian(FluidDomain& d, MyFloat dt) { step(d, FS_STEP_SEMI_LAGRANGIAN, dt); }
void FluidSolver::stepPIC(FluidDomain& d, MyFloat dt) { step(d, FS_STEP_PIC, dt); }
void FluidSolver::stepFLIP(FluidDomain& d, MyFloat dt) { step(d, FS_STEP_FLIP, dt); }
void FluidSolver::stepPICFLIP(FluidDomain& d, MyFloat dt) { step(d, FS_STEP_PICFLIP, dt); }
