"""MCPL output and input components: scattering done on the host between
the device halves of the component's pass (ramp_component_enter/leave),
so the neutron state is seen, as in the reference, in the component's own
frame.  Plain path only (the whole-chain kernels never stop mid-chain)."""
import numpy as np
import torch

from .sprim import SPrim
from .. import _abi, mcpl

SE2V = 437.393377
# lanes gathered for output, in ascending lane order: x y z vx vy vz px py pz p tof
_OUT_LANES = sum(1 << l for l in range(11))


class SMCPLOut(SPrim):
    """Dump every neutron not flagged dead (die lane != 1) at this point of
    the chain into an MCPL file (mcpl_out.py:56-103).  The records are
    compacted on the device in index order (ramp_gather_alive) and copied
    once to the host.  The file is rewritten for every chunk, as the
    reference does.  packing="ramp" writes RAMP's own layout byte for byte;
    "mcpl" the standard direction packing (ramp_gb300.mcpl)."""
    kind = _abi.S_HOST

    def __init__(self, filename="", packing="ramp", idx=0, ctx=0, **kwargs):
        self.filename = filename
        self.packing = packing
        self.last_count = 0

    def host_action(self, inst, st, n):
        lib = inst._lib()
        dev = inst.device
        out = torch.empty((max(n, 1), 11), dtype=torch.float32, device=dev)
        scratch = torch.empty(max(1, (n + 1023) // 1024), dtype=torch.int64, device=dev)
        count = torch.zeros(1, dtype=torch.int64, device=dev)
        stream = inst._stream_ptr()
        _abi.check(lib, lib.ramp_gather_alive(_abi.ctypes.byref(st), n, _OUT_LANES,
                                              _abi.ctypes.c_void_p(out.data_ptr()),
                                              _abi.ctypes.c_void_p(scratch.data_ptr()),
                                              scratch.numel(),
                                              _abi.ctypes.c_void_p(count.data_ptr()), stream),
                   "ramp_gather_alive")
        k = int(count.item())
        rows = out[:k].cpu().numpy()
        mcpl.write(self.filename, rows[:, 0:3], rows[:, 3:6], rows[:, 6:9], rows[:, 10],
                   rows[:, 9], packing=self.packing)
        self.last_count = k


class SMCPLIn(SPrim):
    """Replace the neutron buffer with the particles of an MCPL file
    (mcpl_in.py:9-77): position cm -> m, velocity = direction *
    sqrt(E[meV]) * 437.393377, time ms -> s, weight, polarisation, RNG
    counter randint(0, 2^30) + index from NumPy's global generator; indices
    past the file's particles are dead.  A file with more particles than the
    chunk fills the chunk (the reference stops with an index error)."""
    kind = _abi.S_HOST

    def __init__(self, filename="", idx=0, ctx=0, **kwargs):
        self.filename = filename
        self._data = None

    def host_action(self, inst, st, n):
        if self._data is None:
            self._data = mcpl.read(self.filename)
        d = self._data
        m = min(n, len(d["x"]))
        lanes = np.zeros((_abi.NLANES, n), dtype=np.float32)
        ke = d["ekin"][:m] * 1e9
        lanes[0] = np.pad(d["x"][:m] * 1e-2, (0, n - m))
        lanes[1] = np.pad(d["y"][:m] * 1e-2, (0, n - m))
        lanes[2] = np.pad(d["z"][:m] * 1e-2, (0, n - m))
        for l, k in ((3, "ux"), (4, "uy"), (5, "uz")):
            lanes[l, :m] = d[k][:m] * np.sqrt(ke) * SE2V
        for l, k in ((6, "polx"), (7, "poly"), (8, "polz")):
            lanes[l, :m] = d[k][:m]
        lanes[9, :m] = d["weight"][:m]
        lanes[10, :m] = d["time"][:m] * 1e-3
        lanes[11, :m] = (np.random.randint(0, 2 ** 30, size=m) + np.arange(m)).astype(np.float32)
        lanes[15, m:] = 1.0
        inst.state[:, :n].copy_(torch.from_numpy(lanes))
