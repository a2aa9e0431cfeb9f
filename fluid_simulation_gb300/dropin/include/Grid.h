// Drop-in for the reference's include/Grid.h: GridInterface (sizes, deltas,
// index transforms), Grid<T> (a host grid with the reference's bilinear
// sample and splat) and BBox.  These are plain host containers, as in the
// reference; the simulation state itself lives on the GPU (see MacGrid.h).
#ifndef GRID_H
#define GRID_H

#include <cassert>
#include <vector>

#include "MathDefinitions.h"

class GridInterface
{
public:
    GridInterface(int size_x, int size_y, MyFloat delta_x = 1, MyFloat delta_y = 1)
        : _SIZE_X(size_x), _SIZE_Y(size_y), _DELTA_X(delta_x), _DELTA_Y(delta_y)
    {
    }

    inline void linearTo2D(int idx, int* i, int* j) const
    {
        *i = idx % _SIZE_X;
        *j = idx / _SIZE_X;
    }
    inline int twoDToLinear(int i, int j) const
    {
        assert(indexIsValid(i, j));
        return i + j * _SIZE_X;
    }
    inline void worldToCell(MyFloat x, MyFloat y, int* i, int* j) const
    {
        *i = x / _DELTA_X;
        *j = y / _DELTA_Y;
    }
    inline void cellToWorld(int i, int j, MyFloat* x, MyFloat* y) const
    {
        assert(indexIsValid(i, j));
        *x = i * _DELTA_X;
        *y = j * _DELTA_Y;
    }
    inline bool indexIsValid(int i, int j) const { return i >= 0 && i < _SIZE_X && j >= 0 && j < _SIZE_Y; }

    inline int sizeX() const { return _SIZE_X; }
    inline int sizeY() const { return _SIZE_Y; }
    inline MyFloat deltaX() const { return _DELTA_X; }
    inline MyFloat deltaY() const { return _DELTA_Y; }
    inline MyFloat lengthX() const { return _SIZE_X * _DELTA_X; }
    inline MyFloat lengthY() const { return _SIZE_Y * _DELTA_Y; }

protected:
    int _SIZE_X;
    int _SIZE_Y;
    MyFloat _DELTA_X;
    MyFloat _DELTA_Y;
};

template <class T>
class Grid : public GridInterface
{
public:
    Grid(int size_x, int size_y, MyFloat delta_x = 1, MyFloat delta_y = 1)
        : GridInterface(size_x, size_y, delta_x, delta_y), data(static_cast<size_t>(size_x) * size_y, T())
    {
    }

    inline T value(int i, int j) const { return data[twoDToLinear(i, j)]; }
    inline T& operator()(int i, int j) { return data[twoDToLinear(i, j)]; }

    // Bilinear sample at world (x, y): truncated cell index, clamped
    // neighbours (the +1 neighbour after clamping), x then y.
    inline T valueInterpolated(MyFloat x, MyFloat y) const
    {
        int i = x / _DELTA_X, j = y / _DELTA_Y;
        const MyFloat fi = x / _DELTA_X - i, fj = y / _DELTA_Y - j;
        i = CLAMP(i, 0, _SIZE_X - 1);
        j = CLAMP(j, 0, _SIZE_Y - 1);
        const int i1 = CLAMP(i + 1, 0, _SIZE_X - 1), j1 = CLAMP(j + 1, 0, _SIZE_Y - 1);
        const MyFloat a = (1 - fi) * value(i, j) + fi * value(i1, j);
        const MyFloat b = (1 - fi) * value(i, j1) + fi * value(i1, j1);
        return (1 - fj) * a + fj * b;
    }

    // Bilinear splat of `v` at world (x, y): the +1 neighbours are formed
    // before clamping, corners written in the order 00, 10, 01, 11.
    inline void addToValueInterpolated(MyFloat x, MyFloat y, T v)
    {
        int i = x / _DELTA_X, j = y / _DELTA_Y;
        int i1 = i + 1, j1 = j + 1;
        const MyFloat fi = x / _DELTA_X - i, fj = y / _DELTA_Y - j;
        i = CLAMP(i, 0, _SIZE_X - 1);
        j = CLAMP(j, 0, _SIZE_Y - 1);
        i1 = CLAMP(i1, 0, _SIZE_X - 1);
        j1 = CLAMP(j1, 0, _SIZE_Y - 1);
        const MyFloat v0 = (1 - fj) * v, v1 = fj * v;
        (*this)(i, j) += (1 - fi) * v0;
        (*this)(i1, j) += fi * v0;
        (*this)(i, j1) += (1 - fi) * v1;
        (*this)(i1, j1) += fi * v1;
    }

    // Raw storage (row-major i + j * sizeX), used by the GPU mirrors.
    inline T* raw() { return data.data(); }
    inline const T* raw() const { return data.data(); }

protected:
    std::vector<T> data;
};

template <class T>
struct BBox
{
    T x_min, x_max, y_min, y_max;
};

#endif
