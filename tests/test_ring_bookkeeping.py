"""Slot bookkeeping of the TMA tile rings (heatsim2_gb300/csrc/hs2g_ring.h), compiled with g++ and run on the CPU.

The y / z sweeps keep copies in flight in a ring of mbarrier slots and wait on each slot with a bounded wait.
When a wait gives up, the CTA aborts and must still wait for every copy it has in flight before it exits, on
the phase those copies will complete.  This checks that a slot whose wait timed out stays pending at its phase,
and that completed waits advance the slot.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "heatsim2_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include "hs2g_ring.h"
using hs2g::SlotRing;
#define CHECK(c) do { if (!(c)) { std::printf("FAIL line %d: %s\n", __LINE__, #c); return 1; } } while (0)
int main() {
  // two slots, the producer issues tiles 0 and 1
  SlotRing r;
  r.issued(0);
  r.issued(1);
  CHECK(r.in_flight(0) && r.in_flight(1));
  CHECK(r.phase(0) == 0 && r.phase(1) == 0);
  // tile 0 completes: slot 0 advances to phase 1 and is free; tile 2 goes into slot 0
  r.waited(0, true);
  CHECK(!r.in_flight(0) && r.phase(0) == 1);
  r.issued(0);
  // the wait for tile 1 gives up: slot 1 stays pending on phase 0, the phase its copies will complete
  r.waited(1, false);
  CHECK(r.in_flight(1) && r.phase(1) == 0);
  CHECK(r.in_flight(0) && r.phase(0) == 1);
  // the abort drain visits exactly the slots with copies in flight, each on its pending phase
  int drained = 0;
  for (int s = 0; s < 2; ++s)
    if (r.in_flight(s)) drained |= 1 << s;
  CHECK(drained == 3);
  // a completed drain wait clears the slot
  r.waited(1, true);
  CHECK(!r.in_flight(1) && r.phase(1) == 1);
  // many rounds on one slot alternate its phase
  SlotRing q;
  for (int round = 0; round < 9; ++round) {
    CHECK(q.phase(5) == (uint32_t)(round & 1));
    q.issued(5);
    q.waited(5, true);
  }
  CHECK(q.pending == 0);
  std::printf("ok\n");
  return 0;
}
"""


def test_timed_out_slot_stays_pending_for_the_drain(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "ring_test.cpp"
    exe = tmp_path / "ring_test"
    src.write_text(PROGRAM)
    subprocess.check_call([gxx, "-std=c++17", "-O1", "-I" + CSRC, str(src), "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == "ok"
