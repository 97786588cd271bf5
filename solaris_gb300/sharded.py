"""One system's sinks partitioned over the ranks of a process group.

RungeKutta4::Driver (Solaris/RungeKutta4.cpp:20-57, Step :58-129) for a
system too large for one GPU's time budget: rank r owns the contiguous block
of bodies [lo_r, hi_r) (replicas.shard).  Per stage each rank

  1. forms its block's stage input y0 + h (a k) in the reference's operation
     order,
  2. all-gathers every block's positions (24 N bytes in all) into its copy
     of the full state,
  3. evaluates the forces on its own sinks against every source
     (sol_accel_sinks_device: the loop over i of GravityAC,
     Acceleration.cpp:248-329, restricted to the block),

and the step's result is formed per block.  A step's only exchanges are the
four all-gathers of positions (the first of them is the previous step's
result).  RK4 has no error norm; no other reduction is needed.  Every
operation is elementwise on the block or the reference's own force
arithmetic, so the concatenated blocks are the single-GPU RK4 driver's state
bit for bit (checked with gloo ranks on the CPU, tests/test_cpu_sharded.py).

The force backend is pluggable: DeviceSinks (the CUDA kernels, NCCL-ready
device tensors) in production; tests substitute a CPU backend.
"""
from __future__ import annotations

import numpy as np

from . import replicas

A = (0.5, 0.5, 1.0)                        # a21, a32, a43
B = (1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0)  # b1..b4
C = (0.0, 0.5, 0.5, 1.0)                   # c1..c4


class DeviceSinks:
    """Forces of one rank's sinks on the device: a heliocentric context of
    the whole system whose pair kernels run over the block only.  Tensors
    are torch CUDA tensors on the context's stream."""

    def __init__(self, system, lo: int, hi: int, device: int = 0, precision: int = 0):
        import torch

        from . import engine
        self.torch = torch
        self.ctx = engine.Context(system, device=device, precision=precision)
        self.lo, self.hi = lo, hi
        self.dev = torch.device("cuda", device)
        self.stream = torch.cuda.ExternalStream(self.ctx.stream_handle(), device=self.dev)
        self.dydt = torch.zeros(6 * system.n, dtype=torch.float64, device=self.dev)

    def zeros(self, n):
        return self.torch.zeros(n, dtype=self.torch.float64, device=self.dev)

    def accel(self, t: float, y_all):
        """dydt rows [lo, hi) as a (hi - lo, 6) view."""
        from . import abi
        lib = self.ctx.lib
        abi.check(lib, lib.sol_accel_sinks_device(self.ctx.h, float(t), y_all.data_ptr(), self.lo, self.hi,
                                                  self.dydt.data_ptr()))
        return self.dydt.view(-1, 6)[self.lo:self.hi]

    def close(self):
        self.ctx.close()


class ShardedRK4:
    """RK4 driver calls of one system whose sinks are split over the ranks
    of the default process group (or a single process when there is none)."""

    def __init__(self, system, backend_factory=None, device: int = 0, precision: int = 0):
        rank, world = _rank_world()
        self.rank, self.world = rank, world
        self.n = system.n
        self.bounds = [replicas.shard(system.n, r, world) for r in range(world)]
        self.lo, self.hi = self.bounds[rank]
        if backend_factory is None:
            self.be = DeviceSinks(system, self.lo, self.hi, device=device, precision=precision)
        else:
            self.be = backend_factory(system, self.lo, self.hi)
        self.y_all = self.be.zeros(6 * system.n)
        self.y0 = self.be.zeros(6 * (self.hi - self.lo))

    def set_state(self, y0_full):
        """Every rank passes the full initial state; each keeps its block."""
        y = np.ascontiguousarray(y0_full, dtype=np.float64)
        block = y[6 * self.lo:6 * self.hi]
        with self._stream():
            self._assign(self.y0, block)
            self._assign(self.y_all, y)

    def get_state(self):
        """The full state (every rank's block), gathered on every rank."""
        with self._stream():
            parts = self._all_gather_rows(self.y0.reshape(-1, 6), 6)
            return np.asarray(_to_numpy(parts)).reshape(-1)

    def step(self, t: float, h: float, n_steps: int = 1):
        """n_steps RungeKutta4::Driver calls (fixed h); returns the time."""
        with self._stream():
            return self._steps(t, h, n_steps)

    def _stream(self):
        """Device backends: every tensor operation and collective on the
        context's stream, in order with its kernels."""
        stream = getattr(self.be, "stream", None)
        if stream is None:
            import contextlib
            return contextlib.nullcontext()
        return self.be.torch.cuda.stream(stream)

    def _steps(self, t, h, n_steps):
        for _ in range(n_steps):
            k1 = self._eval(t + C[0] * h, self.y0)   # RungeKutta4::Driver: accel at y0
            k1 = _copy(k1)
            k2 = _copy(self._eval(t + C[1] * h, self.y0 + h * (A[0] * k1)))
            k3 = _copy(self._eval(t + C[2] * h, self.y0 + h * (A[1] * k2)))
            k4 = self._eval(t + C[3] * h, self.y0 + h * (A[2] * k3))
            y = self.y0 + h * (B[0] * k1 + B[1] * k2 + B[2] * k3 + B[3] * k4)
            self._assign(self.y0, y)
            t = t + h
        return t

    # -- internals ---------------------------------------------------------------
    def _eval(self, t, y_block):
        """All-gather the block's positions into the full state, then the
        forces of this rank's sinks (flattened (6 (hi - lo),))."""
        yb = y_block.reshape(-1, 6)
        pos = self._all_gather_rows(yb[:, :3], 3)
        ya = self.y_all.reshape(-1, 6)
        ya[:, :3] = pos
        ya[self.lo:self.hi, 3:] = yb[:, 3:]
        return self.be.accel(t, self.y_all).reshape(-1)

    def _all_gather_rows(self, rows, width):
        """Concatenation of every rank's rows (blocks of uneven size)."""
        if self.world == 1:
            return rows
        import torch
        import torch.distributed as dist
        t = rows if isinstance(rows, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(rows))
        n_max = max(hi - lo for lo, hi in self.bounds)
        buf = torch.zeros((n_max, width), dtype=torch.float64, device=t.device)
        buf[: t.shape[0]] = t
        out = [torch.empty_like(buf) for _ in range(self.world)]
        dist.all_gather(out, buf)
        full = torch.cat([o[: hi - lo] for o, (lo, hi) in zip(out, self.bounds)])
        return full if isinstance(rows, torch.Tensor) else full.numpy()

    def _assign(self, dst, src):
        if isinstance(dst, np.ndarray):
            dst[:] = src
        else:
            dst.copy_(src if not isinstance(src, np.ndarray) else self.be.torch.from_numpy(src))

    def close(self):
        close = getattr(self.be, "close", None)
        if close:
            close()


def _rank_world():
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            return dist.get_rank(), dist.get_world_size()
    except ImportError:
        pass
    return 0, 1


def _copy(a):
    return a.copy() if isinstance(a, np.ndarray) else a.clone()


def _to_numpy(a):
    return a if isinstance(a, np.ndarray) else a.detach().cpu().numpy()
