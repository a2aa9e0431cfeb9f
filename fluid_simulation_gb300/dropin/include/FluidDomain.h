// Drop-in for the reference's include/FluidDomain.h.  A FluidDomain owns one
// fsgpu handle: its MacGrid and MarkerParticleSet are mirrors of the grid
// and particles that live on the GPU.  Fluid sources are registered with the
// handle and spawn their particles on the device (fs_update), appended to the
// device set in the reference's order.
#ifndef FLUID_DOMAIN_H
#define FLUID_DOMAIN_H

#include <vector>

#include <LevelSet.h>
#include <MacGrid.h>
#include <MarkerParticleSet.h>

#include "MathDefinitions.h"

class FluidSource
{
public:
    FluidSource(BBox<MyFloat> area, MyFloat delta_x, MyFloat delta_y, MyFloat x_velocity, MyFloat y_velocity,
                MyFloat time_step, int max_spawns);
    ~FluidSource();
    void update(MarkerParticleSet& particle_set, MyFloat dt);
    inline bool isFinished() { return _max_spawns != -1 && _n_spawns >= _max_spawns; }
    inline void resetSpawns() { _n_spawns = 0; }

private:
    BBox<MyFloat> _area;
    MyFloat _x_velocity, _y_velocity, _delta_x, _delta_y, _time_step, _time_since_last;
    int _max_spawns, _n_spawns;
    friend class FluidDomain;  // not in the reference: hands the source to the device
};

class FluidDomain : public GridInterface
{
public:
    FluidDomain(int size_x, int size_y, MyFloat length_x, MyFloat length_y, MyFloat density, MyFloat pic_ratio);
    ~FluidDomain();
    FluidDomain(const FluidDomain&) = delete;
    FluidDomain& operator=(const FluidDomain&) = delete;

    void addFluidSource(FluidSource fluid_source);
    void update(MyFloat dt);
    void clearFluidSources();
    void resetParticleSet();
    void setPicRatio(MyFloat pic_ratio);

    MacGrid& macGrid();
    LevelSet& levelSet();
    MarkerParticleSet& markerParticleSet();
    const MacGrid& macGrid() const;
    const LevelSet& levelSet() const;
    const MarkerParticleSet& markerParticleSet() const;
    const MyFloat density() const;
    const MyFloat picRatio() const;

    void advectLevelSet(MyFloat dt);
    void classifyCells(LevelSet& levelSet);
    void classifyCells(MarkerParticleSet& particle_set);

    // ---- not in the reference: the GPU state behind this domain
    fs_handle* handle() const { return _h; }
    void pushToDevice();     // upload host changes before GPU work
    void deviceUpdated();    // GPU work changed grid and particles

private:
    fs_handle* _h;
    MyFloat _density;
    MyFloat _pic_ratio;
    MacGrid _mac_grid;
    LevelSet _level_set;
    MarkerParticleSet _particle_set;
    std::vector<FluidSource> _fluid_sources;
};

#endif
