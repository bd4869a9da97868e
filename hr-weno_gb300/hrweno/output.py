"""Output-time snapshots: the example drivers' text files, written without stalling the GPU.

The reference's examples write, at every output time, the state as one text record
(example/example1_burgers_1d_fv.f90:153-177, example/example2_pbe_2d_fv.f90:188-217):

    x.txt   header "(a5, 2(1x, a15))": i, x(i), dx(i); rows "(i5, 2(1x, es15.5))"
            (2D: x1.txt and x2.txt, one per direction)
    u.txt   header "(a16)" t, then "(1x, a16)" u(1) ... ; rows "(es16.5e3)" t, "(1x, es16.5e3)" u(i)
            over the whole state (2D: u((j-1) n1 + i)); every record is closed by the
            list-directed write of "" (:169, :177), which puts one blank before the record ends

SnapshotWriter copies each device state into a device slot on the producing stream (an HBM-speed
copy, after which the state may change again), then to a pinned host slot on a side stream
that overlaps the next integration, and formats the records on a worker thread, so a driver
loop over output times keeps the GPU busy.
"""
from __future__ import annotations

import math
import queue
import threading
from pathlib import Path

import numpy as np


def fortran_es(x: float, w: int, d: int, e: int | None = None) -> str:
    """Fortran ESw.d[Ee] edit descriptor: one nonzero digit before the point, d after it,
    exponent with e digits (default: 2, or 3 when it does not fit), right-justified in w."""
    x = float(x)
    if math.isnan(x):
        s = "NaN"
    elif math.isinf(x):
        s = "-Infinity" if x < 0 else "Infinity"
        if len(s) > w:
            s = "-Inf" if x < 0 else "Inf"
    else:
        if x == 0.0:
            mant, ex = "0." + "0" * d, 0
        else:
            m, ex_s = f"{abs(x):.{d}E}".split("E")
            mant, ex = m, int(ex_s)
        sign = "-" if (x < 0 or (x == 0.0 and math.copysign(1.0, x) < 0)) else ""
        es = "+" if ex >= 0 else "-"
        if e is None and abs(ex) > 99:  # ESw.d without Ee: the letter E gives way to a digit
            s = f"{sign}{mant}{es}{abs(ex):03d}"
        else:
            s = f"{sign}{mant}E{es}{abs(ex):0{e if e is not None else 2}d}"
    return s.rjust(w) if len(s) <= w else "*" * w


def fortran_a(text: str, w: int) -> str:
    """Fortran Aw output: right-justified in w (truncated to the leftmost w characters)."""
    return text.rjust(w) if len(text) <= w else text[:w]


def write_grid(path: Path, centers, widths) -> None:
    """x.txt of the examples."""
    lines = [fortran_a("i", 5) + " " + fortran_a("x(i)", 15) + " " + fortran_a("dx(i)", 15)]
    for i, (c, w) in enumerate(zip(centers, widths), start=1):
        lines.append(f"{i:5d}" + " " + fortran_es(c, 15, 5) + " " + fortran_es(w, 15, 5))
    Path(path).write_text("\n".join(lines) + "\n")


def u_header(n: int) -> str:
    return (fortran_a("t", 16) + "".join(" " + fortran_a(f"u({i})", 16) for i in range(1, n + 1))
            + " ")


def u_record(t: float, u) -> str:
    return fortran_es(t, 16, 5, 3) + "".join(" " + fortran_es(v, 16, 5, 3) for v in u) + " "


class SnapshotWriter:
    """Asynchronous u.txt writer: snapshot(t, u) returns at once.

    grids: one (centers, widths) pair per direction; a single direction writes x.txt, several
    write x1.txt, x2.txt, ...; the state holds the product of their sizes."""

    def __init__(self, folder, grids, depth: int = 4):
        import torch
        self.folder = Path(folder)
        self.folder.mkdir(parents=True, exist_ok=True)
        self.n = 1
        for d, (centers, widths) in enumerate(grids, start=1):
            name = "x.txt" if len(grids) == 1 else f"x{d}.txt"
            write_grid(self.folder / name, centers, widths)
            self.n *= len(centers)
        self._fh = open(self.folder / "u.txt", "w")
        self._fh.write(u_header(self.n) + "\n")
        self._slots = [torch.empty(self.n, dtype=torch.float64).pin_memory() for _ in range(depth)]
        self._dev = [torch.empty(self.n, dtype=torch.float64, device="cuda") for _ in range(depth)]
        self._free: queue.Queue = queue.Queue()
        for k in range(depth):
            self._free.put(k)
        self._work: queue.Queue = queue.Queue()
        self._error: BaseException | None = None  # the worker's failure, raised in the caller
        self._copy = torch.cuda.Stream()
        self._thread = threading.Thread(target=self._run, daemon=True)
        self._thread.start()

    def snapshot(self, t: float, u, stream=None) -> None:
        """Queue the state u (CUDA float64 tensor) at time t; the copy is ordered after the work
        already queued on `stream` (default: the current stream)."""
        import torch
        self._raise()
        k = self._free.get()  # waits only when `depth` snapshots are still being written
        self._raise()
        prod = stream or torch.cuda.current_stream()
        with torch.cuda.stream(prod):
            self._dev[k].copy_(u)  # ordered before any later work on the producing stream
        ev = torch.cuda.Event()
        ev.record(prod)
        with torch.cuda.stream(self._copy):
            self._copy.wait_event(ev)
            self._slots[k].copy_(self._dev[k], non_blocking=True)
            done = torch.cuda.Event()
            done.record(self._copy)
        self._work.put((t, k, done))

    def _run(self) -> None:
        while True:
            item = self._work.get()
            if item is None:
                return
            t, k, done = item
            try:
                done.synchronize()
                if self._error is None:
                    self._fh.write(u_record(t, self._slots[k].numpy()) + "\n")
            except BaseException as e:  # noqa: BLE001 - handed to the caller
                self._error = e
            self._free.put(k)  # a waiting snapshot() wakes up and raises

    def _raise(self) -> None:
        if self._error is not None:
            raise RuntimeError("snapshot writer failed") from self._error

    def close(self) -> None:
        self._work.put(None)
        self._thread.join()
        self._fh.close()
        self._raise()
