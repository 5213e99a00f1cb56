"""gpuRIR's own CUDA kernels run on this GPU as a parity oracle.  Test
infrastructure only: nothing in the gpurir_gb300 package imports this module.

build_ref() compiles the device code of the reference's unmodified
src/gpuRIR_cuda.cu, where it lies in the reference checkout, into
oracle/_ref/gpuRIR_ref.cubin with the flags of the reference's CMakeLists.txt
(-D_FORCE_INLINES; Release: -O3 -DNDEBUG) for sm_103a.  Only device code is
compiled, so the cubin carries no host object and runs wherever a GB300 is.

RefKernels loads that cubin through the CUDA driver API (libcuda via ctypes, in
the context torch made current) and replays the host side of
cuda_simulateRIR (src/gpuRIR_cuda.cu:766-931) around the reference's kernels:
the same kernels, launch geometry, buffer shapes and reduction ladder
(cuda_rirGenerator :618-674, cuda_rirGenerator_mp :676-734, the texture table
of create_sinc_texture_lut :574-611).  The host replay is written here; every
number on the device comes from the reference's own kernels.  cuRAND is not
replayed: the diffuse stage takes caller-supplied uniforms (diffRev_kernel
:445-461 transforms whatever the buffer holds).
"""
import ctypes
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, "_ref")
CUBIN = os.path.join(REF_DIR, "gpuRIR_ref.cubin")
# The reference checkout (given to build_ref, or by GPURIR_REFERENCE_ROOT); the
# recipe below reads src/gpuRIR_cuda.cu there.
REF_ROOT = os.environ.get("GPURIR_REFERENCE_ROOT")

# Itanium-mangled names of the reference kernels (signatures at
# src/gpuRIR_cuda.cu:245, 377, 392, 415, 445, 492, 515, 541, 559).
K_AMPTAU = "_Z17calcAmpTau_kernelPfS_S_S_S_S_S_iifffffffffiiiiiff"
K_GEN = "_Z18generateRIR_kernelPfS_S_iiiiif"
K_RED = "_Z16reduceRIR_kernelPfS_iiii"
K_ENV = "_Z14envPred_kernelPfS_S_S_iiiffffffffff"
K_DIFF = "_Z14diffRev_kernelPfS_S_S_iiii"
K_GEN_MP = "_Z21generateRIR_mp_kernelP7__half2PfS1_iiiiiffS_"
K_RED_MP = "_Z19reduceRIR_mp_kernelP7__half2S0_iiii"
K_H2F = "_Z24h2RIR_to_floatRIR_kernelP7__half2Pfii"
K_GEN_LUT = "_Z22generateRIR_kernel_lutPfS_S_iiiiiiyf"

# Launch constants of the reference host code (src/gpuRIR_cuda.cu:20-40).
_ISM_BLOCK = (4, 4, 4)
_INI_RED_MIN = 512
_GEN_BLOCK = (32, 4, 1)
_RED_THREADS = 128
_ENV_BLOCK = (4, 4, 1)
_DIFF_BLOCK = (16, 4, 2)
_LUT_OVERSAMP = 16


def build_ref(root=None, force=False):
    """Compile the reference's device code into oracle/_ref/gpuRIR_ref.cubin.

    `root` is the reference checkout (default: $GPURIR_REFERENCE_ROOT).  Returns
    the cubin path, or None when the checkout is absent (the cubin built
    earlier, if any, is then used as is)."""
    root = root or REF_ROOT
    src = os.path.join(root, "src", "gpuRIR_cuda.cu") if root else ""
    if not src or not os.path.exists(src):
        return CUBIN if os.path.exists(CUBIN) else None
    if not force and os.path.exists(CUBIN) and os.path.getmtime(CUBIN) >= os.path.getmtime(src):
        return CUBIN
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = CUBIN + ".tmp%d" % os.getpid()
    cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-D_FORCE_INLINES",
           "-O3", "-DNDEBUG", "-o", tmp, src]
    subprocess.check_call(cmd, cwd=REF_DIR)
    os.replace(tmp, CUBIN)
    return CUBIN


def available():
    return os.path.exists(CUBIN)


def _ceil_f32(a, b):
    """ceil((float)a / b) in float32, as the reference sizes its grids."""
    return int(math.ceil(float(np.float32(a) / np.float32(b))))


class _ArrayDesc(ctypes.Structure):       # CUDA_ARRAY_DESCRIPTOR
    _fields_ = [("Width", ctypes.c_size_t), ("Height", ctypes.c_size_t),
                ("Format", ctypes.c_int), ("NumChannels", ctypes.c_uint)]


class _ResDesc(ctypes.Structure):         # CUDA_RESOURCE_DESC (128-byte union)
    _fields_ = [("resType", ctypes.c_int), ("res", ctypes.c_uint64 * 16), ("flags", ctypes.c_uint)]


class _TexDesc(ctypes.Structure):         # CUDA_TEXTURE_DESC
    _fields_ = [("addressMode", ctypes.c_int * 3), ("filterMode", ctypes.c_int),
                ("flags", ctypes.c_uint), ("maxAnisotropy", ctypes.c_uint),
                ("mipmapFilterMode", ctypes.c_int), ("mipmapLevelBias", ctypes.c_float),
                ("minMipmapLevelClamp", ctypes.c_float), ("maxMipmapLevelClamp", ctypes.c_float),
                ("borderColor", ctypes.c_float * 4), ("reserved", ctypes.c_int * 12)]


_CU_AD_FORMAT_FLOAT = 0x20
_CU_TR_ADDRESS_MODE_BORDER = 3
_CU_TR_FILTER_MODE_LINEAR = 1
_CU_RESOURCE_TYPE_ARRAY = 0


class RefKernels:
    """The reference's kernels in the current torch CUDA context."""

    def __init__(self, cubin=None):
        import torch
        cubin = cubin or CUBIN
        if not os.path.exists(cubin):
            raise FileNotFoundError("reference cubin missing: %s (run oracle.ref_kernels.build_ref())"
                                    % cubin)
        self.torch = torch
        torch.cuda.init()
        torch.empty(1, device="cuda")          # make the primary context current
        cu = ctypes.CDLL("libcuda.so.1")
        vp, u, sz = ctypes.c_void_p, ctypes.c_uint, ctypes.c_size_t
        cu.cuGetErrorName.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        cu.cuCtxGetCurrent.argtypes = [ctypes.POINTER(vp)]
        cu.cuModuleLoad.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p]
        cu.cuModuleUnload.argtypes = [vp]
        cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
        cu.cuLaunchKernel.argtypes = [vp, u, u, u, u, u, u, u, vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
        cu.cuCtxSynchronize.argtypes = []
        cu.cuArrayCreate_v2.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(_ArrayDesc)]
        cu.cuArrayDestroy.argtypes = [vp]
        cu.cuMemcpyHtoA_v2.argtypes = [vp, sz, vp, sz]
        cu.cuTexObjectCreate.argtypes = [ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(_ResDesc),
                                         ctypes.POINTER(_TexDesc), vp]
        cu.cuTexObjectDestroy.argtypes = [ctypes.c_ulonglong]
        self.cu = cu
        ctx = vp()
        self._ck(cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self.module = vp()
        self._ck(cu.cuModuleLoad(ctypes.byref(self.module), cubin.encode()), "cuModuleLoad")
        self.fn = {}
        for name in (K_AMPTAU, K_GEN, K_RED, K_ENV, K_DIFF, K_GEN_MP, K_RED_MP, K_H2F, K_GEN_LUT):
            f = vp()
            self._ck(cu.cuModuleGetFunction(ctypes.byref(f), self.module, name.encode()), name)
            self.fn[name] = f

    def _ck(self, rc, what):
        if rc != 0:
            s = ctypes.c_char_p()
            self.cu.cuGetErrorName(rc, ctypes.byref(s))
            raise RuntimeError("%s failed: %s (%d)" % (what, (s.value or b"?").decode(), rc))

    def _launch(self, name, grid, block, shmem, args):
        objs = [ct(v) for ct, v in args]
        params = (ctypes.c_void_p * len(objs))(*[ctypes.addressof(o) for o in objs])
        self._ck(self.cu.cuLaunchKernel(self.fn[name], grid[0], grid[1], grid[2], block[0], block[1],
                                        block[2], shmem, None, params, None), name)
        self._ck(self.cu.cuCtxSynchronize(), name)

    def _dev(self, a, dtype=None):
        t = self.torch
        if a is None:
            return None
        return t.from_numpy(np.ascontiguousarray(a, dtype=dtype or np.float32)).cuda()

    def _empty(self, n, dtype=None):
        return self.torch.zeros(max(int(n), 1), dtype=dtype or self.torch.float32, device="cuda")

    # -- cuda_rirGenerator, src/gpuRIR_cuda.cu:618-674 ---------------------------------
    def _rir_generator(self, rir, amp, tau, M, N, T, Fs, lut):
        P = ctypes.c_void_p
        I, F = ctypes.c_int, ctypes.c_float
        ini_red = _INI_RED_MIN
        while float(np.float32(M * T) * np.float32(_ceil_f32(N, ini_red))) > 1e9:
            ini_red *= 2
        ini_n = _ceil_f32(N, ini_red)
        grid = (_ceil_f32(T, _GEN_BLOCK[0]), _ceil_f32(M, _GEN_BLOCK[1]), ini_n)
        initial = self._empty(M * T * ini_n)
        Tw = _window_len(Fs)
        if lut:
            lut_len = Tw * _LUT_OVERSAMP
            lut_len += 0 if lut_len % 2 else 1
            import oracle
            table = np.ascontiguousarray(oracle.lut_table(Fs), dtype=np.float32)
            assert table.size == lut_len
            arr = ctypes.c_void_p()
            desc = _ArrayDesc(lut_len, 0, _CU_AD_FORMAT_FLOAT, 1)
            self._ck(self.cu.cuArrayCreate_v2(ctypes.byref(arr), ctypes.byref(desc)), "cuArrayCreate")
            tex = ctypes.c_ulonglong()
            try:
                self._ck(self.cu.cuMemcpyHtoA_v2(arr, 0, table.ctypes.data, table.nbytes), "cuMemcpyHtoA")
                rd = _ResDesc()
                rd.resType = _CU_RESOURCE_TYPE_ARRAY
                rd.res[0] = arr.value
                td = _TexDesc()
                # only addressMode[0] is set, the others stay 0 (wrap) as after the
                # reference's memset: a 1D fetch also filters along y at y = 0, and a
                # border there would blend in half a texel of the zero border colour
                td.addressMode[0] = _CU_TR_ADDRESS_MODE_BORDER
                td.filterMode = _CU_TR_FILTER_MODE_LINEAR
                self._ck(self.cu.cuTexObjectCreate(ctypes.byref(tex), ctypes.byref(rd), ctypes.byref(td),
                                                   None), "cuTexObjectCreate")
                self._launch(K_GEN_LUT, grid, _GEN_BLOCK, 0,
                             [(P, initial.data_ptr()), (P, amp.data_ptr()), (P, tau.data_ptr()),
                              (I, T), (I, M), (I, N), (I, ini_n), (I, ini_red), (I, Tw // 2),
                              (ctypes.c_ulonglong, tex.value), (F, lut_len // 2 + 0.5)])
            finally:
                if tex.value:
                    self.cu.cuTexObjectDestroy(tex)
                self.cu.cuArrayDestroy(arr)
        else:
            self._launch(K_GEN, grid, _GEN_BLOCK, 0,
                         [(P, initial.data_ptr()), (P, amp.data_ptr()), (P, tau.data_ptr()),
                          (I, T), (I, M), (I, N), (I, ini_n), (I, ini_red), (F, float(Tw))])
        red_block = (_RED_THREADS, 1, 1)
        while ini_n > 2 * _RED_THREADS:
            int_n = _ceil_f32(ini_n, 2 * _RED_THREADS)
            inter = self._empty(int_n * T * M)
            self._launch(K_RED, (int_n, T, M), red_block, _RED_THREADS * 4,
                         [(P, initial.data_ptr()), (P, inter.data_ptr()), (I, M), (I, T), (I, ini_n),
                          (I, int_n)])
            initial, ini_n = inter, int_n
        self._launch(K_RED, (1, T, M), red_block, _RED_THREADS * 4,
                     [(P, initial.data_ptr()), (P, rir.data_ptr()), (I, M), (I, T), (I, ini_n), (I, 1)])

    # -- cuda_rirGenerator_mp, src/gpuRIR_cuda.cu:676-734 -------------------------------
    def _rir_generator_mp(self, rir, amp, tau, M, N, T, Fs):
        P = ctypes.c_void_p
        I, F = ctypes.c_int, ctypes.c_float
        ini_red = _INI_RED_MIN
        while float(np.float32((M * T) // 2) * np.float32(_ceil_f32(N, ini_red))) > 1e9:
            ini_red *= 2
        ini_n = _ceil_f32(N, ini_red)
        Th = T // 2
        grid = (int(math.ceil(float(np.float32(T) / np.float32(2) / np.float32(_GEN_BLOCK[0])))),
                _ceil_f32(M, _GEN_BLOCK[1]), ini_n)
        h2 = self.torch.int32
        initial = self._empty(M * Th * ini_n, h2)
        fs32 = np.float32(Fs)
        tw_2 = float(np.float32(8e-3) * fs32 / np.float32(2))
        tw_inv = np.float16(np.float32(1.0) / (np.float32(8e-3) * fs32))
        h2_tw_inv = int(np.array([tw_inv, tw_inv], dtype=np.float16).view(np.uint32)[0])
        self._launch(K_GEN_MP, grid, _GEN_BLOCK, 0,
                     [(P, initial.data_ptr()), (P, amp.data_ptr()), (P, tau.data_ptr()), (I, Th),
                      (I, M), (I, N), (I, ini_n), (I, ini_red), (F, float(fs32)), (F, tw_2),
                      (ctypes.c_uint32, h2_tw_inv)])
        red_block = (_RED_THREADS, 1, 1)
        while ini_n > 2 * _RED_THREADS:
            int_n = _ceil_f32(ini_n, 2 * _RED_THREADS)
            inter = self._empty(int_n * Th * M, h2)
            self._launch(K_RED_MP, (int_n, Th, M), red_block, _RED_THREADS * 4,
                         [(P, initial.data_ptr()), (P, inter.data_ptr()), (I, M), (I, Th), (I, ini_n),
                          (I, int_n)])
            initial, ini_n = inter, int_n
        inter = self._empty(M * Th, h2)
        self._launch(K_RED_MP, (1, Th, M), red_block, _RED_THREADS * 4,
                     [(P, initial.data_ptr()), (P, inter.data_ptr()), (I, M), (I, Th), (I, ini_n), (I, 1)])
        self._launch(K_H2F, (_ceil_f32(Th, 128), M, 1), (128, 1, 1), 0,
                     [(P, inter.data_ptr()), (P, rir.data_ptr()), (I, M), (I, Th)])

    # -- cuda_simulateRIR, src/gpuRIR_cuda.cu:766-931 -----------------------------------
    def simulate(self, room_sz, beta, pos_src, pos_rcv, nb_img, Tmax, fs, Tdiff=None,
                 spkr_pattern=0, mic_pattern=0, orV_src=None, orV_rcv=None, c=343.0, mode="fp32",
                 uniforms=None, host=True):
        """Early part, envelope and (with `uniforms`, [M_src, M_rcv, nSamples - nSamplesISM]
        float32 in (0, 1), numpy or a CUDA tensor) the diffuse tail, by the reference's
        kernels.  `mode` is "fp32", "mp" (activateMixedPrecision) or "lut" (activateLUT).
        host=False returns the device tensors and copies nothing back."""
        P = ctypes.c_void_p
        I, F = ctypes.c_int, ctypes.c_float
        room = np.asarray(room_sz, dtype=np.float32).reshape(3)
        b = np.asarray(beta, dtype=np.float32).reshape(6)
        ps = np.ascontiguousarray(pos_src, dtype=np.float32).reshape(-1, 3)
        pr = np.ascontiguousarray(pos_rcv, dtype=np.float32).reshape(-1, 3)
        ms, mr = ps.shape[0], pr.shape[0]
        os_ = np.zeros_like(ps) if orV_src is None else np.asarray(orV_src, np.float32).reshape(ms, 3)
        or_ = np.zeros_like(pr) if orV_rcv is None else np.asarray(orV_rcv, np.float32).reshape(mr, 3)
        nb = [int(x) for x in np.asarray(nb_img).reshape(3)]
        N = nb[0] * nb[1] * nb[2]
        M = ms * mr
        Tdiff = Tmax if Tdiff is None else Tdiff
        d_ps, d_pr, d_os, d_or = self._dev(ps), self._dev(pr), self._dev(os_), self._dev(or_)
        amp, tau, tau_dp = self._empty(M * N), self._empty(M * N), self._empty(M)
        shm = ((ms if spkr_pattern == 0 else 2 * ms) + (mr if mic_pattern == 0 else 2 * mr)) * 3 * 4
        grid = tuple(_ceil_f32(nb[d], _ISM_BLOCK[d]) for d in range(3))
        self._launch(K_AMPTAU, grid, _ISM_BLOCK, shm,
                     [(P, amp.data_ptr()), (P, tau.data_ptr()), (P, tau_dp.data_ptr()),
                      (P, d_ps.data_ptr()), (P, d_pr.data_ptr()), (P, d_os.data_ptr()),
                      (P, d_or.data_ptr()), (I, int(spkr_pattern)), (I, int(mic_pattern))] +
                     [(F, float(v)) for v in room] + [(F, float(v)) for v in b] +
                     [(I, nb[0]), (I, nb[1]), (I, nb[2]), (I, ms), (I, mr), (F, float(np.float32(c))),
                      (F, float(np.float32(fs)))])
        n_ism = _n_samples(Tdiff, fs)
        n_tot = _n_samples(Tmax, fs)
        n_diff = n_tot - n_ism
        rir = self._empty(M * n_ism)
        if mode == "mp":
            self._rir_generator_mp(rir, amp, tau, M, N, n_ism, fs)
        else:
            self._rir_generator(rir, amp, tau, M, N, n_ism, fs, lut=(mode == "lut"))
        A, alpha = self._empty(M), self._empty(M)
        self._launch(K_ENV, (_ceil_f32(ms, _ENV_BLOCK[0]), _ceil_f32(mr, _ENV_BLOCK[1]), 1), _ENV_BLOCK, 0,
                     [(P, A.data_ptr()), (P, alpha.data_ptr()), (P, rir.data_ptr()), (P, tau_dp.data_ptr()),
                      (I, ms), (I, mr), (I, n_ism), (F, float(np.float32(fs)))] +
                     [(F, float(v)) for v in room] + [(F, float(v)) for v in b])
        out = dict(amp=amp, tau=tau, tau_dp=tau_dp, early=rir, A=A, alpha=alpha)
        if uniforms is not None and n_diff > 0:
            if isinstance(uniforms, np.ndarray):
                diff = self._dev(np.ascontiguousarray(uniforms, dtype=np.float32).reshape(-1))
            else:
                diff = uniforms.reshape(-1)
            assert diff.numel() == M * n_diff and diff.dtype == self.torch.float32 and diff.is_cuda
            grid = (_ceil_f32(n_diff, _DIFF_BLOCK[0]), _ceil_f32(ms, _DIFF_BLOCK[1]), _ceil_f32(mr, _DIFF_BLOCK[2]))
            self._launch(K_DIFF, grid, _DIFF_BLOCK, 0,
                         [(P, diff.data_ptr()), (P, A.data_ptr()), (P, alpha.data_ptr()),
                          (P, tau_dp.data_ptr()), (I, ms), (I, mr), (I, n_ism), (I, n_diff)])
            out["diffuse"] = diff
        shapes = dict(amp=(ms, mr, N), tau=(ms, mr, N), tau_dp=(ms, mr), early=(ms, mr, n_ism),
                      A=(ms, mr), alpha=(ms, mr), diffuse=(ms, mr, n_diff))
        if host:
            out = {k: v.cpu().numpy().reshape(shapes[k]) for k, v in out.items()}
        out.update(n_ism=n_ism, n_samples=n_tot)
        return out

    def close(self):
        if self.module.value:
            self.cu.cuModuleUnload(self.module)
            self.module = ctypes.c_void_p()


def _n_samples(T, fs):
    """ceil(T*Fs) in float32, rounded up to even (src/gpuRIR_cuda.cu:831-835)."""
    n = int(math.ceil(float(np.float32(T) * np.float32(fs))))
    return n + n % 2


def _window_len(fs):
    """(int) round(8e-3f * Fs) (src/gpuRIR_cuda.cu:628)."""
    return int(math.floor(float(np.float32(8e-3) * np.float32(fs)) + 0.5))


def hash_uniforms(n):
    """Deterministic uniforms in (0, 1) for the diffuse stage: a multiplicative
    hash of the index on 24 bits, (h + 0.5) / 2^24 (exact in float32)."""
    i = np.arange(int(n), dtype=np.uint64)
    h = (i * np.uint64(2654435761)) % np.uint64(1 << 24)
    return ((h.astype(np.float64) + 0.5) / float(1 << 24)).astype(np.float32)
