"""Host-side mirror of the reference's time-stepping interface, on the CUDA C-ABI.

The method names and argument meanings follow the Fortran routines they replace:

================  =====================================  ==============================
method            reference                              C-ABI
================  =====================================  ==============================
``fft_dir(z)``    src/fft_dir.f90:1-24                   ``gt_fft_dir``
``fft_inv(z)``    src/fft_inv.f90:1-16                   ``gt_fft_inv``
``trunc(z)``      src/trunc.f90:1-28                     ``gt_trunc``
``produ(z,u,v)``  src/produ.f90:1-26                     ``gt_produ``
``nlt(z,u,v)``    src/nlt.f90:1-66                       ``gt_nlt``
``step(...)``     src/rkstep.f90:2-76                    ``gt_step_rk2``
``step4(...)``    src/rkstep.f90:82-131                  ``gt_step_rk4``
``forcing(z,s)``  src/forcing.f90:1-36                   ``gt_forcing``
``diag(z,znl)``   src/diagnostics.f90 spectrum/fluxes/glob  ``gt_diag``
================  =====================================  ==============================

Fields are CUDA float64 tensors of shape (N, N+2) (the physical view ``real(8) z(N+2,N)``);
``spec(z)`` is the complex (N, N/2+1) view of the same memory. Work is enqueued on the
solver's stream (the current torch stream at construction unless one is given).
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np
import torch

from . import _lib
from .params import GtInfo, Params


def _tune_cache_default() -> str:
    """Autotuner cache: $GTURBO_TUNE_CACHE, else autotune.json beside the built library."""
    return os.environ.get("GTURBO_TUNE_CACHE") or os.path.join(os.path.dirname(_lib.LIB_PATH),
                                                               "autotune.json")


def _read_cache(path: str | None) -> dict:
    if path is None or not os.path.exists(path):
        return {}
    try:
        with open(path) as f:
            table = json.load(f)
        return table if isinstance(table, dict) else {}
    except (OSError, ValueError):
        return {}


def _write_cache(path: str, table: dict) -> None:
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def spec(z: torch.Tensor) -> torch.Tensor:
    """Complex (NY, NX/2+1) view of an (NY, NX+2) float64 field."""
    return z.view(torch.complex128).view(z.shape[0], z.shape[1] // 2)


class Solver:
    """One parameter set on one device: tables, forced modes and the hot-path routines."""

    def __init__(self, p: Params, device: int | torch.device | None = None,
                 stream: torch.cuda.Stream | None = None):
        self.lib = _lib.load()
        self.p = p
        self.n = p.n  # NX
        self.ny = p.rows  # NY
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else
                                   torch.device(device).index or 0)
        self._cp = p.to_ctypes()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            torch.cuda.init()
            rc = self.lib.gt_create(ctypes.byref(self._cp), ctypes.byref(h))
            if rc != 0:
                raise _lib.GturboError(rc, self.lib.gt_last_error(None).decode())
        self.h = h
        self.stream = stream if stream is not None else torch.cuda.current_stream(self.device)
        self._check(self.lib.gt_set_stream(self.h, ctypes.c_void_p(self.stream.cuda_stream)))
        info = GtInfo()
        self._check(self.lib.gt_get_info(self.h, ctypes.byref(info)))
        self.info = info
        self.nf = info.nf

    # -- bookkeeping ---------------------------------------------------------------------
    def _check(self, rc: int) -> None:
        _lib.check(self.lib, self.h, rc)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.gt_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field(self) -> torch.Tensor:
        return torch.zeros((self.ny, self.n + 2), dtype=torch.float64, device=self.device)

    def work(self, count: int = 4) -> list[torch.Tensor]:
        return [self.field() for _ in range(count)]

    def _ptr(self, t: torch.Tensor) -> int:
        if t.dtype != torch.float64 or not t.is_cuda or not t.is_contiguous():
            raise ValueError("fields must be contiguous float64 CUDA tensors")
        if t.numel() != (self.n + 2) * self.ny:
            raise ValueError(f"field has {t.numel()} values, expected (NX+2)*NY = {(self.n + 2) * self.ny}")
        return t.data_ptr()

    def forcing_modes(self):
        ik = (ctypes.c_int32 * 2048)()
        jk = (ctypes.c_int32 * 2048)()
        nf = ctypes.c_int32()
        self._check(self.lib.gt_get_forcing_modes(self.h, ik, jk, ctypes.byref(nf)))
        return np.array(ik[:nf.value], np.int32), np.array(jk[:nf.value], np.int32)

    def sync(self) -> None:
        self._check(self.lib.gt_sync(self.h))

    PROF_KINDS = ("nlt_colinv", "nlt_row", "nlt_colfwd", "forcing", "diag", "other",
                  "nlt_colfwd_inv")

    def profile(self, enable: bool) -> None:
        """Record CUDA events around every later launch (gt_profile)."""
        self._check(self.lib.gt_profile(self.h, 1 if enable else 0))

    def profile_read(self) -> dict:
        """{kind: (total ms, launches)} since the last read (gt_profile_read)."""
        ms = (ctypes.c_double * 7)()
        cnt = (ctypes.c_int64 * 7)()
        self._check(self.lib.gt_profile_read(self.h, ms, cnt))
        return {k: (ms[i], cnt[i]) for i, k in enumerate(self.PROF_KINDS)}

    # -- launch variants (gt_set_variant / gt_autotune) -----------------------------------
    NVARIANTS = 6

    @property
    def variant(self) -> int:
        v = ctypes.c_int32()
        self._check(self.lib.gt_get_variant(self.h, ctypes.byref(v)))
        return v.value

    @variant.setter
    def variant(self, v: int) -> None:
        self._check(self.lib.gt_set_variant(self.h, int(v)))

    @property
    def variants(self) -> tuple[int, int]:
        """(column variant, row variant) of the handle."""
        c, r = ctypes.c_int32(), ctypes.c_int32()
        self._check(self.lib.gt_get_variants(self.h, ctypes.byref(c), ctypes.byref(r)))
        return c.value, r.value

    @variants.setter
    def variants(self, cr) -> None:
        self._check(self.lib.gt_set_variants(self.h, int(cr[0]), int(cr[1])))

    @property
    def col_split(self) -> int:
        """The field-split column passes that run (gt_get_col_split): 0 none, 1 pass C's epilogue
        by the column's second CTA, 2 pass C as 2-CTA clusters sharing the epilogue."""
        a = ctypes.c_int32()
        self._check(self.lib.gt_get_col_split(self.h, ctypes.byref(a)))
        return a.value

    @col_split.setter
    def col_split(self, mode: int) -> None:
        self._check(self.lib.gt_set_col_split(self.h, int(mode)))

    @property
    def pdl(self) -> bool:
        """Whether the pass kernels launch with programmatic dependent launch (gt_get_pdl)."""
        a = ctypes.c_int32()
        self._check(self.lib.gt_get_pdl(self.h, ctypes.byref(a)))
        return bool(a.value)

    @pdl.setter
    def pdl(self, on: bool) -> None:
        self._check(self.lib.gt_set_pdl(self.h, int(bool(on))))

    @property
    def graphs(self) -> bool:
        """Whether the steps replay CUDA graphs of the handle (gt_get_graphs)."""
        a = ctypes.c_int32()
        self._check(self.lib.gt_get_graphs(self.h, ctypes.byref(a)))
        return bool(a.value)

    @graphs.setter
    def graphs(self, on: bool) -> None:
        self._check(self.lib.gt_set_graphs(self.h, int(bool(on))))

    @property
    def adj_memory(self) -> int:
        """Device memory (bytes) the adjoint gradient may hold for whole kept segments
        (gt_adj_get_memory; 0 = only its last segment)."""
        a = ctypes.c_int64()
        self._check(self.lib.gt_adj_get_memory(self.h, ctypes.byref(a)))
        return int(a.value)

    @adj_memory.setter
    def adj_memory(self, nbytes: int) -> None:
        self._check(self.lib.gt_adj_set_memory(self.h, int(nbytes)))

    def supported_variants(self) -> list[int]:
        ok = [v for v in range(self.NVARIANTS) if self.lib.gt_variant_supported(self.ny, v)]
        return ok if self.ny == self.n else [v for v in ok if v in (1, 2)]

    def supported_row_variants(self) -> list[int]:
        return [r for r in range(self.NVARIANTS) if self.lib.gt_row_variant_supported(self.n, r)]

    def autotune(self, steps: int = 20, cache: str | None = "default") -> dict:
        """Pick the fastest launch variant of the nonlinear-term passes (gt_autotune).

        With a cache file (JSON, keyed by device name, N, integrator order and the library
        file's size and time), a stored choice is reused without timing; None disables it. Returns
        {"variant": column variant, "row_variant": row variant, "col_split": the field-split
        mode that runs (0, 1, 2: ``col_split``), "ms_per_step": per column variant or None,
        "cached": bool}.
        """
        if cache == "default":
            cache = _tune_cache_default()
        # the library's identity (size, mtime) is part of the key: a rebuilt library re-times
        st = os.stat(getattr(self.lib, "_gt_path", _lib.LIB_PATH))
        key = (f"{torch.cuda.get_device_name(self.device)}|n={self.n}"
               f"{'' if self.ny == self.n else 'x' + str(self.ny)}|rko={self.info.rko}"
               f"|lib={st.st_size}-{int(st.st_mtime)}")
        table = _read_cache(cache)
        hit = table.get(key)
        if (hit and hit.get("variant") in self.supported_variants()
                and hit.get("row_variant") in self.supported_row_variants()):
            self.variants = (hit["variant"], hit["row_variant"])
            if "col_split" in hit:
                self.col_split = hit["col_split"]
            return {"variant": hit["variant"], "row_variant": hit["row_variant"],
                    "col_split": self.col_split, "ms_per_step": hit.get("ms_per_step"), "cached": True}
        ms = (ctypes.c_double * self.NVARIANTS)()
        best = ctypes.c_int32()
        self._check(self.lib.gt_autotune(self.h, int(steps), ms, ctypes.byref(best)))
        col, row = self.variants
        split = self.col_split
        res = {"variant": col, "row_variant": row, "col_split": split, "ms_per_step": list(ms),
               "cached": False}
        if cache is not None:
            table[key] = {"variant": col, "row_variant": row, "col_split": split, "ms_per_step": list(ms)}
            _write_cache(cache, table)
        return res

    # -- the reference's routines -----------------------------------------------------------
    def fft_dir(self, z: torch.Tensor) -> None:
        self._check(self.lib.gt_fft_dir(self.h, self._ptr(z)))

    def fft_inv(self, z: torch.Tensor) -> None:
        self._check(self.lib.gt_fft_inv(self.h, self._ptr(z)))

    def dump_real4(self, z: torch.Tensor) -> np.ndarray:
        """The physical field of z as the reference's real(4) dump (src/write.f90:29-51): an
        N x N float32 array (x fastest), inverse-transformed and converted on the device."""
        with torch.cuda.stream(self.stream):
            work = z.clone()
            out = torch.empty((self.ny, self.n), dtype=torch.float32, device=self.device)
        self._check(self.lib.gt_dump_real4(self.h, self._ptr(work), out.data_ptr()))
        with torch.cuda.stream(self.stream):
            host = out.cpu()
        return host.numpy()

    def load_real4(self, w, z: torch.Tensor | None = None) -> torch.Tensor:
        """Restart from a real(4) dump (src/read.f90:3-27 + src/main.f90:89-92): the N x N
        float32 physical field w (numpy or tensor, x fastest) -> spectral field z, fft_dir'ed
        and truncated on the device (gt_load_real4). Returns z."""
        with torch.cuda.stream(self.stream):
            wd = torch.as_tensor(np.ascontiguousarray(w, np.float32) if isinstance(w, np.ndarray) else w)
            wd = wd.to(self.device, torch.float32).contiguous()
            if wd.shape != (self.ny, self.n):
                raise ValueError(f"dump must be {self.ny} x {self.n} float32 (NY rows of NX)")
            if z is None:
                z = self.field()
        # wd was allocated on the solver's stream: its memory is not reused before the
        # kernels enqueued here have read it
        self._check(self.lib.gt_load_real4(self.h, wd.data_ptr(), self._ptr(z)))
        return z

    def trunc(self, z: torch.Tensor) -> None:
        self._check(self.lib.gt_trunc(self.h, self._ptr(z)))

    def produ(self, z, u, v) -> None:
        self._check(self.lib.gt_produ(self.h, self._ptr(z), self._ptr(u), self._ptr(v)))

    def nlt(self, z, u, v) -> None:
        self._check(self.lib.gt_nlt(self.h, self._ptr(z), self._ptr(u), self._ptr(v)))

    def step(self, z, znl, u, v) -> None:
        self._check(self.lib.gt_step_rk2(self.h, self._ptr(z), self._ptr(znl), self._ptr(u), self._ptr(v)))

    def step4(self, z, znl, znew, u, v) -> None:
        self._check(self.lib.gt_step_rk4(self.h, self._ptr(z), self._ptr(znl), self._ptr(znew),
                                         self._ptr(u), self._ptr(v)))

    def rk_step(self, z, work) -> None:
        """``step4`` when rko=4, else ``step`` (src/main.f90:100-104). work = [znl, znew, u, v]."""
        znl, znew, u, v = work
        if self.info.rko == 4:
            self.step4(z, znl, znew, u, v)
        else:
            self.step(z, znl, u, v)

    def rk_step_forced(self, z, work, seed: int) -> int:
        """``rk_step`` followed by ``forcing`` with the kick fused into the final stage
        (gt_step_rk2_forced / gt_step_rk4_forced); returns the LCG state after the kick."""
        znl, znew, u, v = work
        s = ctypes.c_int32(int(seed))
        if self.info.rko == 4:
            self._check(self.lib.gt_step_rk4_forced(self.h, self._ptr(z), self._ptr(znl), self._ptr(znew),
                                                    self._ptr(u), self._ptr(v), ctypes.byref(s)))
        else:
            self._check(self.lib.gt_step_rk2_forced(self.h, self._ptr(z), self._ptr(znl), self._ptr(u),
                                                    self._ptr(v), ctypes.byref(s)))
        return s.value

    def forcing(self, z, seed: int) -> int:
        """Adds one kick; returns the LCG state after the nf draws."""
        s = ctypes.c_int32(int(seed))
        self._check(self.lib.gt_forcing(self.h, self._ptr(z), ctypes.byref(s)))
        return s.value

    def forcing_philox(self, z, key: int, step: int) -> None:
        """The kick with counter-based Philox phases (gt_forcing_philox)."""
        self._check(self.lib.gt_forcing_philox(self.h, self._ptr(z), int(key), int(step)))

    def diag(self, z, znl=None) -> dict:
        """spectrum / fluxes / glob of src/diagnostics.f90 (synchronous)."""
        nb = self.n // 2
        out = {k: np.zeros(nb) for k in ("sp", "sz")}
        glob = np.zeros(6)
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        if znl is not None:
            out["fle"], out["flz"] = np.zeros(nb), np.zeros(nb)
            rc = self.lib.gt_diag(self.h, self._ptr(z), self._ptr(znl), dp(out["sp"]), dp(out["sz"]),
                                  dp(out["fle"]), dp(out["flz"]), dp(glob))
        else:
            rc = self.lib.gt_diag(self.h, self._ptr(z), None, dp(out["sp"]), dp(out["sz"]),
                                  None, None, dp(glob))
        self._check(rc)
        out["glob"] = glob
        return out

    def main_step(self, z, seed: int, work, diag: bool = False):
        """One iteration of src/main.f90:97-137 (step, diagnostics when asked, forcing). The
        diagnostics see the field before the kick, so a diagnostics step keeps the separate
        forcing launch; the others fuse the kick into the step (``rk_step_forced``)."""
        if not diag:
            return self.rk_step_forced(z, work, seed), None
        self.rk_step(z, work)
        znl, _, u, v = work
        with torch.cuda.stream(self.stream):
            znl.copy_(z)
        self.nlt(znl, u, v)
        out = self.diag(z, znl)
        seed = self.forcing(z, seed)
        return seed, out
