// Copy schedule of the CG's pipelined streaming form (k_cg_large in
// fs_cg.cu): how many 1024-cell slots ahead of its use each operand is copied
// into a warp's shared memory with cp.async, the bytes of each ring entry,
// and how many of a thread's copy groups may still be pending at each wait.
// Plain constexpr code: fs_cg.cu compiles it for the device, and the
// schedule's CPU test (tests/test_pipeline_schedule.py) for the host.
#pragma once

#if defined(__CUDACC__)
#define FS_PIPE_HD __host__ __device__
#else
#define FS_PIPE_HD
#endif

namespace fs {
namespace pipe {

// Chunks per CTA from which k_cg_large streams through the pipeline.
constexpr int MIN_CHUNKS = 20;

// Shared-memory layout.  Every warp owns a private WARP_BYTES region and
// copies only the 32 cells it computes (plus the 4-cell pieces around them
// that its edge lanes read), so no copy ever needs a CTA barrier.  Phase A
// keeps PA_STAGES slots of stage 1 (z, p, down, up: 128 bytes each; flags:
// 32; the z and p of the 4 cells before and after the warp's cells: 64) and
// PG_STAGES slots of stage 2 (z and p of each cell's down and up neighbours,
// gathered once its indices have arrived); phase B keeps PB_STAGES slots of z,
// p, x, r, q and flags.  The two phases use the same bytes: each starts after
// the other's copies have all landed.  A slot's entry is reused by the slot
// STAGES later, which is copied once the slot itself has been computed.
constexpr int WARP_BYTES = 6400;
constexpr int PA_ENTRY = 4 * 128 + 32 + 64;
constexpr int PA_STAGES = 6;
constexpr int PA_AHEAD = PA_STAGES - 1;
constexpr int PG_ENTRY = 4 * 128;
constexpr int PG_STAGES = 3;
constexpr int PG_AHEAD = PG_STAGES - 1;
constexpr int PB_ENTRY = 5 * 128 + 32;
constexpr int PB_STAGES = 9;
constexpr int PB_AHEAD = PB_STAGES - 1;
static_assert(PA_STAGES * PA_ENTRY + PG_STAGES * PG_ENTRY <= WARP_BYTES, "phase A stages");
static_assert(PB_STAGES * PB_ENTRY <= WARP_BYTES, "phase B stages");
static_assert(WARP_BYTES % 16 == 0 && PA_ENTRY % 16 == 0 && PG_ENTRY % 16 == 0 && PB_ENTRY % 16 == 0,
              "16-byte copies");
// a CTA of the pipelined form owns at least MIN_CHUNKS - 1 slots
static_assert(MIN_CHUNKS - 1 > PA_AHEAD, "a CTA's last slot is copied after the barrier");

// Phase A's copy groups, in commit order: G1(0..PA_AHEAD-1) (stage 1 of the
// first slots, before the barrier), G2(0..PG_AHEAD-1) (their gathers), then
// per slot k: G2(k + PG_AHEAD), G1(k + PA_AHEAD).  pa_wait1(k): groups
// committed after G1(k + PG_AHEAD) when slot k starts; pa_wait2(k): groups
// committed after G2(k) once slot k's own groups are committed.
FS_PIPE_HD constexpr int pa_wait1(int k)
{
    return k + PG_AHEAD <= PA_AHEAD - 1 ? PA_AHEAD - 1 + k : 2 * (PA_AHEAD - PG_AHEAD - 1);
}
FS_PIPE_HD constexpr int pa_wait2(int k) { return k < PG_AHEAD ? PG_AHEAD + 1 + k : 2 * PG_AHEAD + 1; }
// The wait before slot j's gathers in the post-barrier prologue (j < PG_AHEAD).
constexpr int PA_WAIT_PROLOGUE = PA_AHEAD - 1;
// Slots before both counts settle; from PA_PEEL on the waits are pa_wait*(PA_PEEL).
constexpr int PA_PEEL = 3;
static_assert(PA_PEEL >= PA_AHEAD - PG_AHEAD && PA_PEEL >= PG_AHEAD, "steady waits from slot PA_PEEL on");
static_assert(MIN_CHUNKS - 1 > PA_PEEL, "the peeled slots exist");
// Phase B's groups: GB(0..PB_AHEAD-1) before the barrier, then GB(k +
// PB_AHEAD) per slot k; slot k waits with PB_AHEAD groups pending.
constexpr int PB_WAIT = PB_AHEAD;

}  // namespace pipe
}  // namespace fs
