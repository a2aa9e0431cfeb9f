// Drop-in for the reference's include/MacGrid.h.  The staggered velocity
// grids and cell types live on the GPU (one fsgpu handle per FluidDomain);
// this class keeps host mirrors of them for the reference's inline
// accessors.  A mirror is downloaded on its first read after GPU work and
// uploaded before the next GPU work if a setter changed it, so programs
// written against the reference recompile unchanged (source compatibility;
// the object layout differs from the reference's).
#ifndef MAC_GRID_H
#define MAC_GRID_H

#include <Grid.h>

#include "MathDefinitions.h"

struct fs_handle;

enum CellType
{
    LIQUID,
    AIR,
    SOLID
};

class MacGrid : public GridInterface
{
public:
    MacGrid(int size_x, int size_y, MyFloat length_x, MyFloat length_y);
    ~MacGrid();
    MacGrid(const MacGrid&) = delete;
    MacGrid& operator=(const MacGrid&) = delete;

    void clearCellTypeBuffer();
    void updatePreviousVelocityBuffer();
    void updateVelocityDiffBuffer();

    // Getters (include/MacGrid.h:30-111 of the reference)
    inline MyFloat velX(int i, int j) const { return (rd(UF).value(i, j) + rd(UF).value(i + 1, j)) / 2; }
    inline MyFloat velY(int i, int j) const { return (rd(VF).value(i, j) + rd(VF).value(i, j + 1)) / 2; }
    inline MyFloat velXHalfIndexed(int i, int j) const { return rd(UF).value(i, j); }
    inline MyFloat velYHalfIndexed(int i, int j) const { return rd(VF).value(i, j); }
    inline MyFloat velXBackBufferHalfIndexed(int i, int j) const { return rd(UB).value(i, j); }
    inline MyFloat velYBackBufferHalfIndexed(int i, int j) const { return rd(VB).value(i, j); }
    inline MyFloat velXBackBuffer(int i, int j) const { return (rd(UB).value(i, j) + rd(UB).value(i + 1, j)) / 2; }
    inline MyFloat velYBackBuffer(int i, int j) const { return (rd(VB).value(i, j) + rd(VB).value(i, j + 1)) / 2; }
    inline MyFloat velXInterpolated(MyFloat x, MyFloat y) const { return rd(UF).valueInterpolated(x, y - _DELTA_Y * 0.5); }
    inline MyFloat velYInterpolated(MyFloat x, MyFloat y) const { return rd(VF).valueInterpolated(x - _DELTA_X * 0.5, y); }
    inline MyFloat velXDiffInterpolated(MyFloat x, MyFloat y) const { return rd(UD).valueInterpolated(x, y - _DELTA_Y * 0.5); }
    inline MyFloat velYDiffInterpolated(MyFloat x, MyFloat y) const { return rd(VD).valueInterpolated(x - _DELTA_X * 0.5, y); }
    inline CellType cellType(int i, int j) const
    {
        i = CLAMP(i, 0, _SIZE_X - 1);
        j = CLAMP(j, 0, _SIZE_Y - 1);
        return labels().value(i, j);
    }
    inline MyFloat divVelX(int i, int j) const { return (rd(UF).value(i + 1, j) - rd(UF).value(i, j)) / _DELTA_X; }
    inline MyFloat divVelY(int i, int j) const { return (rd(VF).value(i, j + 1) - rd(VF).value(i, j)) / _DELTA_Y; }

    // Setters (include/MacGrid.h:116-157 of the reference)
    inline void setVelXHalfIndexed(int i, int j, MyFloat v) { wr(UF)(i, j) = v; }
    inline void setVelYHalfIndexed(int i, int j, MyFloat v) { wr(VF)(i, j) = v; }
    inline void setVelXBackBuffer(int i, int j, MyFloat v) { wr(UB)(i, j) = v; wr(UB)(i + 1, j) = v; }
    inline void setVelYBackBuffer(int i, int j, MyFloat v) { wr(VB)(i, j) = v; wr(VB)(i, j + 1) = v; }
    inline void setVelXBackBufferHalfIndexed(int i, int j, MyFloat v) { wr(UB)(i, j) = v; }
    inline void setVelYBackBufferHalfIndexed(int i, int j, MyFloat v) { wr(VB)(i, j) = v; }
    inline void setCellType(int i, int j, CellType t) { labelsW()(i, j) = t; }
    inline void addToVelXInterpolated(MyFloat x, MyFloat y, MyFloat v) { wr(UB).addToValueInterpolated(x, y - 0.5 * _DELTA_Y, v); }
    inline void addToVelYInterpolated(MyFloat x, MyFloat y, MyFloat v) { wr(VB).addToValueInterpolated(x - 0.5 * _DELTA_X, y, v); }

    void swapVelocityBuffers();

    // ---- not in the reference: binding to the GPU state
    void attach(fs_handle* h);  // called by FluidDomain
    void push();                // upload host-modified mirrors before GPU work
    void invalidate();          // GPU work changed the device state

private:
    enum Buf { UF = 0, VF, UB, VB, UP, VP, UD, VD, NBUF };
    const Grid<MyFloat>& rd(Buf b) const;
    Grid<MyFloat>& wr(Buf b);
    const Grid<CellType>& labels() const;
    Grid<CellType>& labelsW();
    void pull(int b) const;

    fs_handle* _h;
    mutable Grid<MyFloat>* _buf[NBUF];
    mutable Grid<CellType> _cell_type_buffer;
    mutable bool _stale[NBUF + 1];  // device newer than the mirror (index NBUF: cell types)
    bool _dirty[NBUF + 1];          // mirror newer than the device
};

#endif
