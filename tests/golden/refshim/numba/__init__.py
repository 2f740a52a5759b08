"""CPU stand-in for the small part of numba's CUDA API that the collocation
reference uses, so that its unmodified Python sources run on a machine without
numba or a GPU.  Used only by ``tests/golden/make_golden.py`` to produce golden
fixtures; nothing in the product imports it.

Semantics reproduced:

* ``@cuda.jit(device=True)`` functions are plain Python functions.
* ``@cuda.jit`` kernels launched as ``kernel[grid, block](*args)`` run every
  (block, thread) pair.  Kernels whose body calls ``cuda.syncthreads`` run each
  block's threads as Python threads with a barrier that releases threads that
  have returned; other kernels run thread by thread.
* ``cuda.shared.array`` returns one NaN-filled array per block and call site
  order; ``cuda.device_array`` returns NaN-filled host arrays so that reads of
  unwritten device memory show up as NaN.
"""
import threading

import numpy as np

float64 = np.float64
int32 = np.int32

_tls = threading.local()


class DeviceNDArray(np.ndarray):
    def copy_to_host(self):
        return np.array(self, copy=True).view(np.ndarray)


def _as_dev(a):
    return np.array(a, copy=True).view(DeviceNDArray)


class _Dim3:
    __slots__ = ("x", "y", "z")

    def __init__(self, x=0, y=0, z=0):
        self.x, self.y, self.z = x, y, z


def _dims(d):
    if isinstance(d, tuple):
        d = tuple(int(v) for v in d) + (1,) * (3 - len(d))
        return d
    return (int(d), 1, 1)


class _Barrier:
    def __init__(self, n):
        self.n = n
        self.waiting = 0
        self.gen = 0
        self.cv = threading.Condition()

    def wait(self):
        with self.cv:
            gen = self.gen
            self.waiting += 1
            if self.waiting >= self.n:
                self.waiting = 0
                self.gen += 1
                self.cv.notify_all()
            else:
                while gen == self.gen:
                    self.cv.wait()

    def leave(self):
        with self.cv:
            self.n -= 1
            if self.n > 0 and self.waiting >= self.n:
                self.waiting = 0
                self.gen += 1
                self.cv.notify_all()


class _BlockState:
    def __init__(self, nthreads):
        self.shared = []
        self.lock = threading.Lock()
        self.barrier = _Barrier(nthreads)


class _Shared:
    @staticmethod
    def array(shape, dtype):
        blk = _tls.block
        idx = _tls.shared_idx
        _tls.shared_idx += 1
        with blk.lock:
            while len(blk.shared) <= idx:
                blk.shared.append(None)
            if blk.shared[idx] is None:
                arr = np.empty(shape, dtype=dtype)
                if np.issubdtype(arr.dtype, np.floating):
                    arr.fill(np.nan)
                blk.shared[idx] = arr
            return blk.shared[idx]


class _Local:
    @staticmethod
    def array(shape, dtype):
        return np.empty(shape, dtype=dtype)


class _Kernel:
    def __init__(self, fn):
        self.fn = fn
        self.uses_sync = "syncthreads" in fn.__code__.co_names

    def __getitem__(self, cfg):
        grid, block = cfg[0], cfg[1]
        g = _dims(grid)
        b = _dims(block)

        def launch(*args):
            self._run(g, b, args)

        return launch

    def _set_thread(self, g, b, bidx, tidx, blk):
        _tls.gridDim = _Dim3(*g)
        _tls.blockDim = _Dim3(*b)
        _tls.blockIdx = _Dim3(*bidx)
        _tls.threadIdx = _Dim3(*tidx)
        _tls.block = blk
        _tls.shared_idx = 0

    def _run(self, g, b, args):
        nthreads = b[0] * b[1] * b[2]
        for bz in range(g[2]):
            for by in range(g[1]):
                for bx in range(g[0]):
                    blk = _BlockState(nthreads)
                    tids = [(tx, ty, tz) for tz in range(b[2]) for ty in range(b[1]) for tx in range(b[0])]
                    if not self.uses_sync:
                        for t in tids:
                            self._set_thread(g, b, (bx, by, bz), t, blk)
                            self.fn(*args)
                        continue
                    errors = []

                    def body(t, bidx=(bx, by, bz)):
                        self._set_thread(g, b, bidx, t, blk)
                        try:
                            self.fn(*args)
                        except BaseException as e:  # pragma: no cover - surfaced below
                            errors.append(e)
                        finally:
                            blk.barrier.leave()

                    ths = [threading.Thread(target=body, args=(t,)) for t in tids]
                    for th in ths:
                        th.start()
                    for th in ths:
                        th.join()
                    if errors:
                        raise errors[0]


class _Cuda:
    shared = _Shared()
    local = _Local()

    @property
    def threadIdx(self):
        return _tls.threadIdx

    @property
    def blockIdx(self):
        return _tls.blockIdx

    @property
    def blockDim(self):
        return _tls.blockDim

    @property
    def gridDim(self):
        return _tls.gridDim

    @staticmethod
    def grid(ndim):
        t, bi, bd = _tls.threadIdx, _tls.blockIdx, _tls.blockDim
        if ndim == 1:
            return bi.x * bd.x + t.x
        if ndim == 2:
            return (bi.x * bd.x + t.x, bi.y * bd.y + t.y)
        return (bi.x * bd.x + t.x, bi.y * bd.y + t.y, bi.z * bd.z + t.z)

    @staticmethod
    def syncthreads():
        _tls.block.barrier.wait()

    @staticmethod
    def to_device(a):
        return _as_dev(a)

    @staticmethod
    def device_array(shape, dtype=np.float64):
        a = np.empty(shape, dtype=dtype)
        if np.issubdtype(a.dtype, np.floating):
            a.fill(np.nan)
        return a.view(DeviceNDArray)

    @staticmethod
    def synchronize():
        return None

    @staticmethod
    def jit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return _Kernel(args[0])
        device = kwargs.get("device", False)

        def deco(fn):
            return fn if device else _Kernel(fn)

        return deco


cuda = _Cuda()


def jit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]):
        return args[0]
    return lambda fn: fn
