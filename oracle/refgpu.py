"""The reference's own FP32 GPU kernel -- TEST INFRASTRUCTURE ONLY.

``kernel`` of 2d/gpumatmult.cu:20-63 (3d/gpumatmult.cu:22-71), compiled unmodified for
sm_103a into oracle/_ref/gpumatmult_{2,3}d.cubin by oracle/build.py (only where the
reference tree is present), loaded here through the CUDA driver API and launched the way
the reference's gpumatmult launches it (2d/gpumatmult.cu:112-115: one 128-thread block per
cell). It is the checker of the library's gpumatmult seam; nothing in the product loads it.

Its last source tile reads up to 127 entries past a block's truncation set
(2d/gpumatmult.cu:50-54), so the source arrays handed to it carry 128 entries of padding.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PAD = 128
# void kernel(int*, float*, float*, float*, float, float*, float*, float*) and the 3D one
# with tZ and sZ, Itanium-mangled
_NAMES = {2: b"_Z6kernelPiPfS0_S0_fS0_S0_S0_", 3: b"_Z6kernelPiPfS0_S0_S0_fS0_S0_S0_S0_"}


def cubin_path(dim):
    return os.path.join(HERE, "_ref", "gpumatmult_%dd.cubin" % dim)


def available(dim):
    return os.path.exists(cubin_path(dim))


class RefKernel:
    def __init__(self, dim):
        import torch
        torch.zeros(1, device="cuda")  # the primary context is current on this thread
        self.torch = torch
        self.dim = dim
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.mod), cubin_path(dim).encode()), "cuModuleLoad")
        self.fn = ctypes.c_void_p()
        self._check(self.cu.cuModuleGetFunction(ctypes.byref(self.fn), self.mod, _NAMES[dim]), "cuModuleGetFunction")

    @staticmethod
    def _check(r, what):
        if r != 0:
            raise RuntimeError("%s failed: CUresult %d" % (what, r))

    def device_args(self, T, S, off, sigma):
        """Device copies: targets (dim arrays of 128 * iblok), sources (dim + 1 arrays,
        padded by PAD zeros), offsets, and the output."""
        t = self.torch
        dev = [t.from_numpy(np.ascontiguousarray(a, np.float32)).cuda() for a in T]
        src = [t.from_numpy(np.concatenate([np.asarray(a, np.float32), np.zeros(PAD, np.float32)])).cuda() for a in S]
        o = t.from_numpy(np.ascontiguousarray(off, np.int32)).cuda()
        w = t.zeros(len(T[0]), dtype=t.float32, device="cuda")
        return dev, src, o, w, np.float32(sigma)

    def launch(self, dev, src, o, w, sigma):
        iblok = o.numel() - 1
        ptr = lambda x: ctypes.c_void_p(x.data_ptr())
        if self.dim == 2:
            vals = [ptr(o), ptr(dev[0]), ptr(dev[1]), ptr(w), ctypes.c_float(sigma), ptr(src[0]), ptr(src[1]), ptr(src[2])]
        else:
            vals = [ptr(o), ptr(dev[0]), ptr(dev[1]), ptr(dev[2]), ptr(w), ctypes.c_float(sigma), ptr(src[0]), ptr(src[1]),
                    ptr(src[2]), ptr(src[3])]
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        stream = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        self._check(self.cu.cuLaunchKernel(self.fn, ctypes.c_uint(iblok), ctypes.c_uint(1), ctypes.c_uint(1),
                                           ctypes.c_uint(128), ctypes.c_uint(1), ctypes.c_uint(1), ctypes.c_uint(0),
                                           stream, params, None), "cuLaunchKernel")

    def __call__(self, T, S, off, sigma):
        args = self.device_args(T, S, off, sigma)
        self.launch(*args)
        self.torch.cuda.synchronize()
        return args[3].cpu().numpy()
