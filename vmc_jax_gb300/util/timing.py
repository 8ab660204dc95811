"""Per-phase GPU timing of the TDVP step with CUDA events on the current
stream, and NVTX ranges of the same phases for profilers (both off unless
enabled; used by the benchmark).  The phases mirror the reference's
start_timing / stop_timing sections of TDVP.__call__ (tdvp.py:256-285)."""

import torch


class PhaseTimer:
    def __init__(self):
        self.enabled = False
        self.nvtx = False
        self.marks = []
        self._open = False

    def reset(self):
        self.marks = []
        self.close()

    def mark(self, name):
        """End the running phase and start ``name`` ("<name>_end" marks only
        end one)."""
        if self.nvtx:
            self.close()
            if not name.endswith("_end"):
                torch.cuda.nvtx.range_push(name)
                self._open = True
        if self.enabled:
            ev = torch.cuda.Event(enable_timing=True)
            ev.record()
            self.marks.append((name, ev))

    def close(self):
        if self._open:
            torch.cuda.nvtx.range_pop()
            self._open = False

    def durations(self):
        """{phase: total ms} where a phase runs from its mark to the next mark
        ("<name>_end" marks close a phase without opening one)."""
        torch.cuda.synchronize()
        out = {}
        for (n0, e0), (n1, e1) in zip(self.marks[:-1], self.marks[1:]):
            if n0.endswith("_end"):
                continue
            out[n0] = out.get(n0, 0.0) + e0.elapsed_time(e1)
        return out

    def spans(self, name):
        """Durations (ms) of every occurrence of ``name`` ... next mark."""
        torch.cuda.synchronize()
        return [e0.elapsed_time(e1) for (n0, e0), (n1, e1) in zip(self.marks[:-1], self.marks[1:]) if n0 == name]


TIMER = PhaseTimer()
