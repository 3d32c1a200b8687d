"""The reference's run loop with its false-vacuum break (main.cpp:77-90),
written against three callables so that the same loop drives the oracle on
the CPU and the library on the GPU:

    for (reset(); tau < TMax; evolve()) {
        Print_AveragesExtrema();            // a row when the TSO cadence is due
        if (false_vacuum_decayed()) break;  // reads the last row's <V>
        ...
    }

Print_AveragesExtrema's cadence (fieldanalysis.cpp:753-780): a row at step 0,
then whenever tau >= LastSOoutput + TSO (LastSOoutput advancing by TSO).
"""
from __future__ import annotations

import ctypes


def decayed_by_library(lib, theory: int):
    """phn_false_vacuum_decayed of the library on a row (26 doubles)."""
    from phinum_gb300 import _lib as L

    def f(row) -> bool:
        a = L.PhnAverages.from_buffer_copy(bytes(memoryview(row.astype("<f8"))))
        d = ctypes.c_int(-1)
        L.check(lib.phn_false_vacuum_decayed(ctypes.byref(a), int(theory), ctypes.byref(d)))
        return bool(d.value)
    return f


def loop_until_decayed(time, averages, evolve1, decayed, nsteps: int, tso: float):
    """Returns (rows, stop): the rows computed and the step count at the
    break, or -1 when the loop ran all nsteps steps."""
    rows, last = [], None
    last_so = 0.0
    for _ in range(nsteps):
        tau, steps = time()
        due = False
        if steps == 0:
            last_so = tau
            due = True
        elif not (tau < last_so + tso):
            if tau >= last_so + tso:
                last_so += tso
            due = True
        if due:
            last = averages()
            last = last.copy()
            last[0] = last_so
            rows.append(last)
        if last is not None and decayed(last):
            return rows, steps
        evolve1()
    return rows, -1
