// Drop-in for the reference's include/MarkerParticleSet.h.  The particles
// live on the GPU; this set is their host mirror.  Appended particles are
// uploaded incrementally; any non-const iteration marks the whole set as
// modified and it is uploaded in full before the next GPU work.
#ifndef PARTICLE_SET_H
#define PARTICLE_SET_H

#include <cstddef>
#include <vector>

#include "MacGrid.h"
#include "MathDefinitions.h"

class MarkerParticle
{
public:
    MarkerParticle() : _pos_x(0), _pos_y(0), _vel_x(0), _vel_y(0) {}
    MarkerParticle(MyFloat pos_x, MyFloat pos_y, MyFloat vel_x = 0, MyFloat vel_y = 0)
        : _pos_x(pos_x), _pos_y(pos_y), _vel_x(vel_x), _vel_y(vel_y)
    {
    }

    inline MyFloat posX() const { return _pos_x; }
    inline MyFloat posY() const { return _pos_y; }
    inline MyFloat velX() const { return _vel_x; }
    inline MyFloat velY() const { return _vel_y; }
    inline void setPosition(MyFloat x, MyFloat y)
    {
        _pos_x = x;
        _pos_y = y;
    }
    inline void setVelocity(MyFloat vx, MyFloat vy)
    {
        _vel_x = vx;
        _vel_y = vy;
    }
    inline void advect(MyFloat dt)
    {
        _pos_x += _vel_x * dt;
        _pos_y += _vel_y * dt;
    }

private:
    // Same 16-byte {x, y, vx, vy} layout as the GPU upload format.
    MyFloat _pos_x, _pos_y, _vel_x, _vel_y;
};

class MarkerParticleSet
{
public:
    MarkerParticleSet(int size = 0);
    ~MarkerParticleSet();

    void addParticle(MarkerParticle p);
    void reserve(int particle_count);
    void clear();
    void advect(MyFloat dt);
    void advectAndEnsureOutsideObstacles(MyFloat dt, const MacGrid& mac_grid);

    typedef std::vector<MarkerParticle>::iterator iterator;
    typedef std::vector<MarkerParticle>::const_iterator const_iterator;

    int size() const;
    iterator begin();
    iterator end();
    const_iterator begin() const;
    const_iterator end() const;

    // ---- not in the reference: binding to the GPU state
    void attach(fs_handle* h);
    void push();
    void invalidate();
    // n particles now on the device (sources appended there); the mirror follows lazily
    void deviceAppended(std::size_t n);

private:
    void pull() const;

    fs_handle* _h;
    mutable std::vector<MarkerParticle> _particles;
    mutable bool _stale;     // device newer than the mirror
    bool _modified;          // mirror changed beyond appends
    std::size_t _synced;     // leading particles already on the device
};

#endif
