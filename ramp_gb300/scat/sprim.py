"""Base class of scattering plugins (mcramp/scat/sprim.py:6-53).

A scattering plugin keeps the reference constructor signature (unknown
keyword arguments are swallowed by ``**kwargs`` as there), writes its
parameters into the scatter slots of a component descriptor (``fill``) and
owns its result buffers as device tensors."""
import torch


def _device(ctx):
    if isinstance(ctx, torch.device):
        return ctx
    if isinstance(ctx, str):
        return torch.device(ctx)
    if isinstance(ctx, int):
        return torch.device("cuda", ctx)
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


class SPrim:
    kind = None

    def fill(self, comp, keep):
        """Write scatter kind and parameters into ``comp`` (a RampComp)."""
        comp.scat = self.kind

    def scatter_prg(self, *args, **kwargs):
        raise NotImplementedError(
            "scattering kernels run fused with their component's geometry kernel; "
            "use Instrument.execute")

    def tallies(self):
        """Device tensors accumulated by this component (for reset/merge)."""
        return []

    def lines(self):
        return [[0], [0], [0]]

    def data_reduce(self, queue):
        return 0

    def data(self, queue):
        return 0

    def plot(self, queue):
        return 0

    def save(self, queue):
        return 0
