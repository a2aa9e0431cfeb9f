// Phases of FluidSolver's step functions over a launch domain (enqueue only).
#include "fs_step.h"

namespace fs {
namespace {

void mark(StepState& st, int k)
{
    if (st.mark) st.mark(st.owner, k);
}

// FluidDomain::classifyCells (src/FluidDomain.cpp:150-180); with_counts:
// also pressureSolve's particle counts (the step's particles do not move
// before its pressure solve).
void ph_classify(const Launch& L, StepState& st, bool with_counts = false)
{
    labels_clear(L, st.d, st.labels);
    if (with_counts) labels_and_counts(L, st.d, st.px, st.py, st.labels, st.counts32, st.warn);
    else labels_from_particles(L, st.d, st.px, st.py, st.labels);
    labels_finalize(L, st.d, st.labels, st.solid);
}

// The two problems of a pair of splats (u faces, then v faces): u on L's
// stream and v on the auxiliary one when the state has it (forked from and
// joined back into L's stream, in a captured graph as outside one), else both
// on L's stream.
template <class U, class V>
void splat_pair(const Launch& L, StepState& st, U u_problem, V v_problem)
{
    if (!st.sw2 || !st.aux) {
        u_problem(L, *st.sw);
        v_problem(L, *st.sw);
        return;
    }
    cudaEventRecord(st.fork, L.stream);
    cudaStreamWaitEvent(st.aux, st.fork, 0);
    Launch La = L;
    La.stream = st.aux;
    u_problem(L, *st.sw);
    v_problem(La, *st.sw2);
    cudaEventRecord(st.join, st.aux);
    cudaStreamWaitEvent(L.stream, st.join, 0);
}

// transferVelocityToGridSpread (src/FluidSolver.cpp:873-919), then the swap.
void ph_p2g(const Launch& L, StepState& st)
{
    p2g_positions(L, st.d, st.px, st.py, st.yu, st.xv);
    splat_pair(
        L, st,
        [&](const Launch& Lu, SplatWork& w) {
            const float* vu[2] = {st.pvx, nullptr};
            float* ou[2] = {st.acc[0], st.acc[1]};
            ordered_splat(Lu, st.d, false, true, st.px, st.yu, nullptr, 2, vu, ou, w);
        },
        [&](const Launch& Lv, SplatWork& w) {
            const float* vv[2] = {st.pvy, nullptr};
            float* ov[2] = {st.acc[2], st.acc[3]};
            ordered_splat(Lv, st.d, false, true, st.xv, st.py, nullptr, 2, vv, ov, w);
        });
    p2g_finish(L, st.d, st.acc[0], st.acc[1], st.acc[2], st.acc[3], st.UB(), st.VB());
    *st.front ^= 1;
}

void ph_save_prev(const Launch& L, StepState& st) { grid_copy2(L, st.d, st.UF(), st.VF(), st.u_prev, st.v_prev); }

void ph_save_diff(const Launch& L, StepState& st)
{
    grid_diff(L, st.d, st.UF(), st.VF(), st.u_prev, st.v_prev, st.u_diff, st.v_diff);
}

void ph_gravity(const Launch& L, StepState& st, float dt) { gravity(L, st.d, st.labels, st.UF(), st.VF(), dt); }

void ph_dirichlet(const Launch& L, StepState& st) { dirichlet(L, st.d, st.labels, st.UF(), st.VF()); }

// extendVelocityIndividual (src/FluidSolver.cpp:485-622), then the swap;
// with_forces: gravity and the Dirichlet condition first, fused with the
// extension's initialisation.
void ph_extend(const Launch& L, StepState& st, bool with_forces = false, float dt = 0.0f)
{
    const int vf = *st.vfront;
    if (with_forces)
        forces_extend_init(L, st.d, st.labels, st.UF(), st.VF(), dt, st.UB(), st.VB(), st.vmx[vf], st.vmx[1 - vf],
                           st.vmy[vf], st.vmy[1 - vf]);
    else
        extend_init(L, st.d, st.labels, st.UF(), st.VF(), st.UB(), st.VB(), st.vmx[vf], st.vmx[1 - vf], st.vmy[vf],
                    st.vmy[1 - vf]);
    for (int it = 0; it < st.n_ext; ++it) {
        const int f = *st.vfront;
        extend_sweep(L, st.d, st.labels, st.UB(), st.VB(), st.vmx[f], st.vmx[1 - f], st.vmy[f], st.vmy[1 - f]);
        *st.vfront ^= 1;
    }
    *st.front ^= 1;
}

// FluidSolver::pressureSolve (src/FluidSolver.cpp:323-483), then the swap;
// counted: the particle counts were taken by the step's classification.
void ph_pressure(const Launch& L, StepState& st, float dt, bool counted = false)
{
    if (!counted) count_particles(L, st.d, st.px, st.py, st.counts32, st.warn);
    fluid_index_batch(L, st.d, st.labels, st.fidx, st.cell_of, st.nfluid, st.index_tmp);
    assemble(L, st.d, st.labels, st.fidx, st.cell_of, st.nfluid, st.UF(), st.VF(), st.cg_b, st.cg_down, st.cg_up,
             st.cg_flags, st.counts32, st.counts8);
    mark(st, FS_T_CG);
    st.solve(st.owner, L);
    mark(st, FS_T_PROJECT);
    project(L, st.d, st.fidx, st.nfluid, st.cg_x, st.UF(), st.VF(), st.UB(), st.VB(), dt);
    *st.front ^= 1;
}

// Grid-to-particle transfer and/or particle advection (one kernel).
void ph_g2p(const Launch& L, StepState& st, int g2p, int adv, float dt)
{
    g2p_advect(L, st.d, g2p, adv, st.px, st.py, st.pvx, st.pvy, st.UF(), st.VF(), st.u_diff, st.v_diff, st.labels,
               dt);
}

// advectVelocitySemiLagrangian (src/FluidSolver.cpp:709-772): no swap.
void ph_sl_velocity(const Launch& L, StepState& st, float dt)
{
    sl_faces(L, st.d, st.labels, st.UF(), st.VF(), dt, st.sl[0], st.sl[1], st.sl[2], st.sl_ok[0], st.sl[3], st.sl[4],
             st.sl[5], st.sl_ok[1]);
    splat_pair(
        L, st,
        [&](const Launch& Lu, SplatWork& w) {
            const float* vu[1] = {st.sl[2]};
            float* ou[1] = {st.UB()};
            ordered_splat(Lu, st.d, true, false, st.sl[0], st.sl[1], st.sl_ok[0], 1, vu, ou, w);
        },
        [&](const Launch& Lv, SplatWork& w) {
            const float* vv[1] = {st.sl[5]};
            float* ov[1] = {st.VB()};
            ordered_splat(Lv, st.d, true, false, st.sl[3], st.sl[4], st.sl_ok[1], 1, vv, ov, w);
        });
}

}  // namespace

void enqueue_phase(const Launch& L, StepState& st, int ph, float dt)
{
    switch (ph) {
        case FS_PH_CLASSIFY: ph_classify(L, st); break;
        case FS_PH_P2G: ph_p2g(L, st); break;
        case FS_PH_SAVE_PREV: ph_save_prev(L, st); break;
        case FS_PH_GRAVITY: ph_gravity(L, st, dt); break;
        case FS_PH_DIRICHLET: ph_dirichlet(L, st); break;
        case FS_PH_EXTEND: ph_extend(L, st); break;
        case FS_PH_PRESSURE: ph_pressure(L, st, dt); break;
        case FS_PH_SAVE_DIFF: ph_save_diff(L, st); break;
        case FS_PH_G2P_PICFLIP: ph_g2p(L, st, G2P_PICFLIP, ADV_NONE, dt); break;
        case FS_PH_G2P_PIC: ph_g2p(L, st, G2P_PIC, ADV_NONE, dt); break;
        case FS_PH_G2P_FLIP: ph_g2p(L, st, G2P_FLIP, ADV_NONE, dt); break;
        case FS_PH_ADVECT_SAFE: ph_g2p(L, st, G2P_NONE, ADV_SAFE, dt); break;
        case FS_PH_ADVECT: ph_g2p(L, st, G2P_NONE, ADV_PLAIN, dt); break;
        case FS_PH_SL_VELOCITY: ph_sl_velocity(L, st, dt); break;
        case FS_PH_SL_PARTICLES: ph_g2p(L, st, G2P_NONE, ADV_RK3, dt); break;
        case FS_PH_SWAP: *st.front ^= 1; break;
        default: break;
    }
}

// FluidSolver::step* (src/FluidSolver.cpp:99-251) as one queued sequence; the
// grid-to-particle transfer and the particle advection share one kernel.
void enqueue_step(const Launch& L, StepState& st, int method, float dt)
{
    mark(st, FS_T_CLASSIFY);
    ph_classify(L, st, true);
    mark(st, FS_T_P2G);
    if (method == FS_STEP_SEMI_LAGRANGIAN) {
        mark(st, FS_T_FORCES);
        ph_sl_velocity(L, st, dt);
        ph_gravity(L, st, dt);
        ph_dirichlet(L, st);
    } else {
        ph_p2g(L, st);
        if (method != FS_STEP_PIC) ph_save_prev(L, st);
        mark(st, FS_T_FORCES);
        ph_extend(L, st, true, dt);  // gravity, Dirichlet, extension
    }
    mark(st, FS_T_ASSEMBLY);
    ph_pressure(L, st, dt, true);
    ph_dirichlet(L, st);
    if (method == FS_STEP_FLIP || method == FS_STEP_PICFLIP) ph_save_diff(L, st);
    mark(st, FS_T_G2P);
    switch (method) {
        case FS_STEP_SEMI_LAGRANGIAN: ph_g2p(L, st, G2P_NONE, ADV_RK3, dt); break;
        case FS_STEP_PIC: ph_g2p(L, st, G2P_PIC, ADV_PLAIN, dt); break;
        case FS_STEP_FLIP: ph_g2p(L, st, G2P_FLIP, ADV_PLAIN, dt); break;
        default: ph_g2p(L, st, G2P_PICFLIP, ADV_SAFE, dt); break;
    }
    mark(st, FS_NUM_TIMED);
}

}  // namespace fs
