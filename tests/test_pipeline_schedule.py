"""The copy schedule of the CG's pipelined streaming form
(fluid_simulation_gb300/csrc/fs_pipeline.h), checked on the host.  The header
is compiled with g++; its constants and wait counts drive a model of one warp
lane's cp.async groups and shared-memory ring entries over whole CG
iterations, for every slot count a CTA of the pipelined form can own:

* every wait completes the groups holding what the next read needs (and no
  more than that: the counts are as large as they may be);
* a copy only goes into a ring entry whose previous slot has been read for
  the last time, and every read finds its own slot in the entry;
* a phase's first copies (into the bytes the other phase's rings used) start
  only when every copy of the other phase has landed.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fluid_simulation_gb300", "csrc")

PROGRAM = r"""
#include "fs_pipeline.h"
#include <cstdio>
int main()
{
    using namespace fs::pipe;
    std::printf("%d %d %d %d %d %d %d %d %d %d\n", MIN_CHUNKS, PA_STAGES, PA_AHEAD, PG_STAGES, PG_AHEAD,
                PB_STAGES, PB_AHEAD, PA_PEEL, PA_WAIT_PROLOGUE, PB_WAIT);
    for (int k = 0; k < 64; ++k) std::printf("%d %d\n", pa_wait1(k), pa_wait2(k));
    return 0;
}
"""


@pytest.fixture(scope="module")
def sched(tmp_path_factory):
    d = tmp_path_factory.mktemp("pipeline_schedule")
    src, exe = d / "schedule.cpp", d / "schedule"
    src.write_text(PROGRAM)
    subprocess.run(["g++", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    lines = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    names = ["min_chunks", "pa_stages", "pa_ahead", "pg_stages", "pg_ahead", "pb_stages", "pb_ahead", "peel",
             "wait_prologue", "pb_wait"]
    s = dict(zip(names, map(int, lines[0].split())))
    s["waits"] = [tuple(map(int, l.split())) for l in lines[1:65]]
    return s


class Lane:
    """One lane's copy groups: commit() closes a group of the copies issued
    since the last commit; wait(n) completes every group but the n most
    recent (cp.async.commit_group / cp.async.wait_group)."""

    def __init__(self):
        self.groups = []
        self.complete = 0
        self.pending = set()

    def copy(self, item):
        self.pending.add(item)

    def commit(self):
        self.groups.append(self.pending)
        self.pending = set()

    def wait(self, n):
        self.complete = max(self.complete, len(self.groups) - n)

    def index(self, item):
        return max(i for i, g in enumerate(self.groups) if item in g)

    def landed(self, item):
        return self.index(item) < self.complete

    def after(self, item):
        return len(self.groups) - 1 - self.index(item)

    def all_landed(self):
        return all(i < self.complete for i, g in enumerate(self.groups) if g)


class Ring:
    """Entries of one ring: which slot each holds, and the slots read for
    the last time."""

    def __init__(self, stages, name):
        self.stages, self.name = stages, name
        self.holds = {}
        self.retired = set()

    def fill(self, slot):
        e = slot % self.stages
        prev = self.holds.get(e)
        assert prev is None or prev in self.retired, (self.name, "entry of slot", prev, "refilled for", slot)
        self.holds[e] = slot

    def read(self, slot):
        assert self.holds.get(slot % self.stages) == slot, (self.name, "entry lost slot", slot)

    def retire(self, slot):
        self.retired.add(slot)

    def reset(self):
        # a phase starts after the other phase's copies have all landed and been read
        self.holds = {}
        self.retired = set()


def run_solve(s, kb, iterations=2):
    """The copies, commits and waits of one lane of k_cg_large's pipelined
    form over `iterations` CG iterations for a CTA owning kb slots."""
    lane = Lane()
    ring_a, ring_g, ring_b = Ring(s["pa_stages"], "stage 1"), Ring(s["pg_stages"], "gathers"), Ring(s["pb_stages"], "phase B")
    pa, pg, pb = s["pa_ahead"], s["pg_ahead"], s["pb_ahead"]

    def stage1(k):
        if k < kb:
            ring_a.fill(k)
            lane.copy(("A1", k))
        lane.commit()

    def gather(k):
        if k < kb:
            assert lane.landed(("A1", k)), ("gathers of slot", k, "before its indices landed")
            ring_a.read(k)
            ring_g.fill(k)
            lane.copy(("G", k))
        lane.commit()

    def prologue_a():
        # the two phases' rings are the same bytes
        assert lane.all_landed(), "phase A copies into bytes that phase B copies may still write"
        ring_a.reset()
        ring_g.reset()
        for k in range(pa):
            stage1(k)

    def prologue_b():
        assert lane.all_landed(), "phase B copies into bytes that phase A copies may still write"
        ring_b.reset()
        for k in range(pb):
            if k < kb:
                ring_b.fill(k)
                lane.copy(("B", k))
            lane.commit()

    prologue_a()  # issued with the initialisation, before its barrier
    for _ in range(iterations):
        for j in range(pg):  # after the barrier
            lane.wait(s["wait_prologue"])
            gather(j)
        for k in range(kb):
            w1, w2 = s["waits"][min(k, s["peel"])]
            lane.wait(w1)
            if k + pg < kb:
                assert lane.after(("A1", k + pg)) == w1, ("slot", k, "wait 1 is not the largest safe count")
            gather(k + pg)
            stage1(k + pa)
            lane.wait(w2)
            assert lane.landed(("A1", k)) and lane.landed(("G", k)), ("slot", k, "read before its copies landed")
            assert lane.after(("G", k)) == w2, ("slot", k, "wait 2 is not the largest safe count")
            ring_a.read(k)
            ring_g.read(k)
            ring_a.retire(k)
            ring_g.retire(k)
        prologue_b()  # before the barrier of p.q
        for k in range(kb):
            if k + pb < kb:
                ring_b.fill(k + pb)
                lane.copy(("B", k + pb))
            lane.commit()
            lane.wait(s["pb_wait"])
            assert lane.landed(("B", k)), ("phase B slot", k, "read before its copies landed")
            assert lane.after(("B", k)) == s["pb_wait"]
            ring_b.read(k)
            ring_b.retire(k)
        prologue_a()  # before the barrier of r.r, r.z
    lane.wait(0)  # cp.async.wait_all before the kernel returns


def test_schedule_constants(sched):
    assert sched["pa_ahead"] == sched["pa_stages"] - 1
    assert sched["pg_ahead"] == sched["pg_stages"] - 1
    assert sched["pb_ahead"] == sched["pb_stages"] - 1
    # the kernel peels slots 0..PA_PEEL-1 and uses the counts of slot PA_PEEL from there on
    steady = sched["waits"][sched["peel"]]
    assert all(w == steady for w in sched["waits"][sched["peel"]:])


@pytest.mark.parametrize("kb", list(range(19, 41)) + [64, 103, 104, 130])
def test_every_wait_and_refill_is_safe(sched, kb):
    # a CTA of the pipelined form owns at least MIN_CHUNKS - 1 slots (4096^2: 103-104)
    assert kb >= sched["min_chunks"] - 1
    run_solve(sched, kb)


def test_model_catches_a_short_wait(sched):
    """The model itself: one pending group too many at slot 3 is reported."""
    bad = dict(sched)
    waits = list(sched["waits"])
    w1, w2 = waits[sched["peel"]]
    waits[sched["peel"]:] = [(w1, w2 + 1)] * (len(waits) - sched["peel"])
    bad["waits"] = waits
    with pytest.raises(AssertionError):
        run_solve(bad, 24, iterations=1)
