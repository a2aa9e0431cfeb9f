// The step sequence of FluidSolver::step* (src/FluidSolver.cpp:99-251) over a
// launch domain: one simulation (fs_handle) or a batch of them (fs_batch).
// Both owners describe their device arrays with a StepState and share the
// phase code below; only the pressure solve differs (a cooperative grid-wide
// CG for one simulation, one thread-block cluster per simulation for a batch).
#pragma once

#include "fs_internal.h"

namespace fs {

struct StepState
{
    Domain d;
    int* front;   // which of u[2], v[2] is the front buffer (MacGrid's swap, a pointer swap)
    int* vfront;  // which of vmx[2], vmy[2] is the front validity mask
    float* u[2];
    float* v[2];
    float *u_prev, *v_prev, *u_diff, *v_diff;
    uint8_t* labels;
    const uint8_t* solid;  // persistent solid mask or nullptr
    uint8_t* vmx[2];
    uint8_t* vmy[2];
    int32_t *fidx, *cell_of, *counts32;
    uint8_t* counts8;
    float* acc[4];
    float* sl[6];
    uint8_t* sl_ok[2];
    float *px, *py, *pvx, *pvy, *yu, *xv;
    SplatWork* sw;
    // With a second scratch, an auxiliary stream and two events, the v
    // problem of each pair of splats runs on aux beside the u problem.
    SplatWork* sw2 = nullptr;
    cudaStream_t aux = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    float* cg_b;
    int32_t *cg_down, *cg_up;
    uint8_t* cg_flags;
    float* cg_x;
    int32_t* nfluid;  // [simulation]
    unsigned* warn;
    int32_t* index_tmp;  // scratch of the fluid indexing
    int n_ext;
    // The pressure solve of the assembled systems, and the per-phase timer mark
    // (k = FS_T_*, FS_NUM_TIMED closes the last phase); mark may be null.
    void (*solve)(void* owner, const Launch& L);
    void (*mark)(void* owner, int k);
    void* owner;

    float* UF() const { return u[*front]; }
    float* VF() const { return v[*front]; }
    float* UB() const { return u[1 - *front]; }
    float* VB() const { return v[1 - *front]; }
};

// FluidSolver::step{SemiLagrangian,PIC,FLIP,PICFLIP} (method = FS_STEP_*).
void enqueue_step(const Launch& L, StepState& st, int method, float dt);
// One reference function (phase = FS_PH_*), for phase-by-phase parity checks.
void enqueue_phase(const Launch& L, StepState& st, int phase, float dt);

}  // namespace fs
