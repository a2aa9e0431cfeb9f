// Multigrid-preconditioned CG for the pressure system (fs_mg.cu): the cell
// grid's own solver, used by the step when the multigrid pressure solver is
// selected and by the standalone Poisson solver's FS_POISSON_MGPCG.
#pragma once

#include "fs_internal.h"

namespace fs {

struct MgSolver;

// Levels and buffers for an nx x ny grid of spacing dx; 0 on success.
int mg_create(MgSolver** out, int nx, int ny, float dx, int device);
void mg_destroy(MgSolver* m);
// The cell types (FS_LIQUID / FS_AIR / FS_SOLID) of the next solves.
void mg_set_labels(MgSolver* m, cudaStream_t st, const uint8_t* labels, int64_t* launches);
// Solves A x = b (the reference's pressure matrix; b one float per cell, read
// on LIQUID cells) to ||r|| < tol ||b||; returns when done.  *x_out points at
// the solution (one float per cell, 0 off LIQUID cells), owned by m.
cudaError_t mg_solve(MgSolver* m, cudaStream_t st, const float* b, double tol, int maxit, int64_t* launches,
                     int* iterations, double* rr, double* bb, float** x_out);

// Right-hand side in fluid-index order -> cells, and the cell solution back.
template <typename T>
void mg_fluid_to_cells(const Launch& L, int64_t ncell, const int32_t* fidx, const int32_t* nfluid, const T* src,
                       float* dst);
template <typename T>
void mg_cells_to_fluid(const Launch& L, int64_t ncell, const int32_t* nfluid, const int32_t* cell_of, const float* src,
                       T* dst);

}  // namespace fs
