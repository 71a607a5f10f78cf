"""Minimal ctypes access to the CUDA runtime (device buffers, pinned host
buffers, events, streams) for the Python mirror, tests and bench. Loads the
same shared libcudart that libgbntt.so links against."""
import ctypes
import ctypes.util
import os

import numpy as np

_rt = None
H2D, D2H, D2D = 1, 2, 3


def rt():
    global _rt
    if _rt is not None:
        return _rt
    cands = ["libcudart.so.13", "libcudart.so", os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"),
                                                           "lib64", "libcudart.so")]
    last = None
    for c in cands:
        try:
            _rt = ctypes.CDLL(c)
            break
        except OSError as e:
            last = e
    if _rt is None:
        raise OSError("libcudart not found: %s" % last)
    R = _rt
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    R.cudaMalloc.argtypes = [ctypes.POINTER(vp), sz]
    R.cudaFree.argtypes = [vp]
    R.cudaMallocHost.argtypes = [ctypes.POINTER(vp), sz]
    R.cudaFreeHost.argtypes = [vp]
    R.cudaMemcpy.argtypes = [vp, vp, sz, ctypes.c_int]
    R.cudaMemcpyAsync.argtypes = [vp, vp, sz, ctypes.c_int, vp]
    R.cudaMemset.argtypes = [vp, ctypes.c_int, sz]
    R.cudaMemsetAsync.argtypes = [vp, ctypes.c_int, sz, vp]
    R.cudaDeviceSynchronize.argtypes = []
    R.cudaStreamSynchronize.argtypes = [vp]
    R.cudaStreamCreate.argtypes = [ctypes.POINTER(vp)]
    R.cudaStreamDestroy.argtypes = [vp]
    R.cudaEventCreate.argtypes = [ctypes.POINTER(vp)]
    R.cudaEventDestroy.argtypes = [vp]
    R.cudaEventRecord.argtypes = [vp, vp]
    R.cudaEventSynchronize.argtypes = [vp]
    R.cudaEventElapsedTime.argtypes = [ctypes.POINTER(ctypes.c_float), vp, vp]
    R.cudaGetErrorString.restype = ctypes.c_char_p
    R.cudaGetErrorString.argtypes = [ctypes.c_int]
    R.cudaGetDeviceCount.argtypes = [ctypes.POINTER(ctypes.c_int)]
    R.cudaDeviceGetAttribute.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int]
    R.cudaMemGetInfo.argtypes = [ctypes.POINTER(sz), ctypes.POINTER(sz)]
    R.cudaSetDevice.argtypes = [ctypes.c_int]
    return R


def check(rc):
    if rc != 0:
        raise RuntimeError("CUDA error %d: %s" % (rc, rt().cudaGetErrorString(rc).decode()))


def device_count():
    n = ctypes.c_int(0)
    return n.value if rt().cudaGetDeviceCount(ctypes.byref(n)) == 0 else 0


def sm_count():
    v = ctypes.c_int(0)
    check(rt().cudaDeviceGetAttribute(ctypes.byref(v), 16, 0))   # cudaDevAttrMultiProcessorCount
    return v.value


def set_device(i):
    check(rt().cudaSetDevice(int(i)))


def mem_info():
    f, t = ctypes.c_size_t(0), ctypes.c_size_t(0)
    check(rt().cudaMemGetInfo(ctypes.byref(f), ctypes.byref(t)))
    return f.value, t.value


class DeviceBuffer:
    def __init__(self, nbytes):
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        check(rt().cudaMalloc(ctypes.byref(p), max(1, self.nbytes)))
        self.ptr = p.value

    def free(self):
        if self.ptr:
            rt().cudaFree(ctypes.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def upload(self, arr, offset=0):
        arr = np.ascontiguousarray(arr)
        assert offset + arr.nbytes <= self.nbytes
        check(rt().cudaMemcpy(ctypes.c_void_p(self.ptr + offset), arr.ctypes.data, arr.nbytes, H2D))

    def download(self, dtype, count, offset=0):
        out = np.empty(count, dtype=dtype)
        assert offset + out.nbytes <= self.nbytes
        check(rt().cudaMemcpy(out.ctypes.data, ctypes.c_void_p(self.ptr + offset), out.nbytes, D2H))
        return out

    def zero(self):
        check(rt().cudaMemset(ctypes.c_void_p(self.ptr), 0, self.nbytes))


class PinnedBuffer:
    """Page-locked host memory viewed as a numpy array."""

    def __init__(self, count, dtype):
        self.dtype = np.dtype(dtype)
        self.nbytes = int(count) * self.dtype.itemsize
        p = ctypes.c_void_p()
        check(rt().cudaMallocHost(ctypes.byref(p), max(1, self.nbytes)))
        self.ptr = p.value
        buf = (ctypes.c_char * max(1, self.nbytes)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(count))

    def free(self):
        if self.ptr:
            self.array = None
            rt().cudaFreeHost(ctypes.c_void_p(self.ptr))
            self.ptr = None


class Event:
    def __init__(self):
        e = ctypes.c_void_p()
        check(rt().cudaEventCreate(ctypes.byref(e)))
        self.ev = e.value

    def record(self, stream=None):
        check(rt().cudaEventRecord(ctypes.c_void_p(self.ev), ctypes.c_void_p(stream) if stream else None))

    def synchronize(self):
        check(rt().cudaEventSynchronize(ctypes.c_void_p(self.ev)))

    def elapsed_ms(self, end):
        ms = ctypes.c_float(0)
        check(rt().cudaEventElapsedTime(ctypes.byref(ms), ctypes.c_void_p(self.ev), ctypes.c_void_p(end.ev)))
        return ms.value


def synchronize():
    check(rt().cudaDeviceSynchronize())


def stream_sync(stream):
    check(rt().cudaStreamSynchronize(ctypes.c_void_p(stream) if stream else None))


def memcpy_async(dst, src, nbytes, kind, stream):
    check(rt().cudaMemcpyAsync(ctypes.c_void_p(dst), ctypes.c_void_p(src), nbytes, kind,
                               ctypes.c_void_p(stream) if stream else None))


def memset_async(ptr, value, nbytes, stream):
    check(rt().cudaMemsetAsync(ctypes.c_void_p(ptr), value, nbytes, ctypes.c_void_p(stream) if stream else None))
