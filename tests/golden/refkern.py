"""Launch PhantomFHE's own CUDA kernels from their cubins through the CUDA driver API.

TEST INFRASTRUCTURE ONLY.  `oracle/Makefile.refgpu` compiles the reference's kernel sources
(unmodified, device code only) into `oracle/_ref/ref_<file>.cubin`; this module loads those
cubins into the current CUDA context (the one torch created), finds each kernel by its
identifier in the cubin's ELF symbol table, checks the arguments against the parameter list
encoded in the mangled name, and launches it with the grid, block and shared-memory sizes the
reference's host code uses.  Device buffers are torch tensors.  Used only by
`make_golden_kernels.py` to produce golden vectors on a GPU; the library never touches it.
"""
import ctypes
import os
import re
import struct

import numpy as np
import torch

REF_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "oracle", "_ref")

_cu = None
# launch mode: stream handle (None = legacy default stream) and whether each launch is
# bracketed by a device synchronisation (always, except while a CUDA graph is being captured)
_mode = {"stream": None, "sync": True}


def set_launch_mode(stream=None, sync=True):
    _mode["stream"], _mode["sync"] = stream, sync


def _driver():
    global _cu
    if _cu is None:
        _cu = ctypes.CDLL("libcuda.so.1")
        _cu.cuModuleLoadData.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        _cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        _cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [ctypes.c_void_p,
                                                                                  ctypes.c_void_p, ctypes.c_void_p]
        _cu.cuCtxSynchronize.argtypes = []
        _cu.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
    return _cu


def _check(rc, what):
    if rc != 0:
        s = ctypes.c_char_p()
        _driver().cuGetErrorString(rc, ctypes.byref(s))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({s.value.decode() if s.value else '?'})")


def elf_function_names(image):
    """Names of the FUNC symbols in an ELF64 image (the kernel entry points of a cubin)."""
    assert image[:4] == b"\x7fELF" and image[4] == 2, "not an ELF64 image"
    shoff, = struct.unpack_from("<Q", image, 0x28)
    shentsize, shnum = struct.unpack_from("<HH", image, 0x3A)
    secs = [struct.unpack_from("<IIQQQQIIQQ", image, shoff + i * shentsize) for i in range(shnum)]
    names = []
    for s in secs:
        if s[1] != 2:  # SHT_SYMTAB
            continue
        stroff = secs[s[6]][4]
        for off in range(s[4], s[4] + s[5], 24):
            name, info = struct.unpack_from("<IB", image, off)
            if info & 0xF == 2:  # STT_FUNC
                names.append(image[stroff + name: image.index(b"\0", stroff + name)].decode())
    return names


def param_sizes(mangled, ident):
    """Byte sizes of the parameters encoded after `ident` in an Itanium-mangled kernel name.
    Covers what these kernels use: pointers (P, with K qualifiers and S..._ substitutions),
    unsigned long (m), unsigned int (j), int (i), double (d)."""
    i = mangled.index(ident) + len(ident)
    if mangled[i] == "E":  # end of a nested name
        i += 1
    sizes = []
    while i < len(mangled):
        ptr = False
        while mangled[i] in "PK":
            ptr |= mangled[i] == "P"
            i += 1
        c = mangled[i]
        if c == "S":
            i = mangled.index("_", i) + 1
            sizes.append(8)  # every substitution used as a parameter here is a pointer type
            continue
        if c.isdigit():
            m = re.match(r"\d+", mangled[i:])
            i += len(m.group(0)) + int(m.group(0))
            assert ptr, f"class passed by value in {mangled}"
            sizes.append(8)
            continue
        i += 1
        sizes.append(8 if ptr else {"m": 8, "j": 4, "i": 4, "d": 8, "y": 8}[c])
    return sizes


class Module:
    def __init__(self, stem):
        path = os.path.join(REF_DIR, f"ref_{stem}.cubin")
        with open(path, "rb") as f:
            self.image = f.read()
        self.names = elf_function_names(self.image)
        self._buf = ctypes.create_string_buffer(self.image, len(self.image))
        self.handle = ctypes.c_void_p()
        _check(_driver().cuModuleLoadData(ctypes.byref(self.handle), ctypes.cast(self._buf, ctypes.c_void_p)),
               f"load {path}")
        self.stem = stem

    def kernel(self, name):
        ident = f"{len(name)}{name}"
        hits = [s for s in self.names if s.startswith("_Z") and re.search(r"(?<!\d)" + ident, s)]
        assert len(hits) == 1, f"{name} in {self.stem}: {hits}"
        f = ctypes.c_void_p()
        _check(_driver().cuModuleGetFunction(ctypes.byref(f), self.handle, hits[0].encode()), name)
        return Kernel(f, name, param_sizes(hits[0], ident))


class Kernel:
    def __init__(self, handle, name, sizes):
        self.handle, self.name, self.sizes = handle, name, sizes

    def __call__(self, grid, block, smem, *args):
        assert len(args) == len(self.sizes), f"{self.name}: {len(args)} args, kernel takes {len(self.sizes)}"
        assert 0 < grid < 2 ** 31 and 0 < block <= 1024 and smem <= 48 * 1024, (self.name, grid, block, smem)
        vals = []
        for a, sz in zip(args, self.sizes):
            if isinstance(a, torch.Tensor):
                assert sz == 8 and a.is_cuda and a.is_contiguous()
                vals.append(ctypes.c_uint64(a.data_ptr()))
            elif isinstance(a, Ptr):
                assert sz == 8
                vals.append(ctypes.c_uint64(a.value))
            elif isinstance(a, float):
                assert sz == 8
                vals.append(ctypes.c_double(a))
            else:
                assert isinstance(a, (int, np.integer)) and a >= 0
                vals.append(ctypes.c_uint64(int(a)) if sz == 8 else ctypes.c_uint32(int(a)))
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        if _mode["sync"]:
            torch.cuda.synchronize()
        _check(_driver().cuLaunchKernel(self.handle, grid, 1, 1, block, 1, 1, smem, _mode["stream"], params, None),
               self.name)
        if _mode["sync"]:
            _check(_driver().cuCtxSynchronize(), self.name)


class Ptr:
    """A device address inside a tensor: `Ptr(t, words)` = t.data_ptr() + 8 * words."""

    def __init__(self, t, words=0):
        assert t.is_cuda and 0 <= words <= t.numel()
        self.value = t.data_ptr() + 8 * words


def dev(a, slack=0):
    """uint64 (or float64) numpy array -> flat int64/float64 CUDA tensor, plus `slack` zero words."""
    a = np.ascontiguousarray(a).reshape(-1)
    if a.dtype == np.float64:
        t = torch.zeros(a.size + slack, dtype=torch.float64)
        t[: a.size] = torch.from_numpy(a)
    else:
        assert a.dtype == np.uint64
        t = torch.zeros(a.size + slack, dtype=torch.int64)
        t[: a.size] = torch.from_numpy(a.view(np.int64))
    return t.cuda()


def host(t, count=None):
    a = t.cpu().numpy().view(np.uint64)
    return a[: count if count is not None else a.size].copy()


def zeros(words):
    return torch.zeros(words, dtype=torch.int64, device="cuda")
