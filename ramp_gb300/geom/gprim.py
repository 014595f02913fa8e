"""Base class of geometry plugins (mcramp/geom/gprim.py:6-28).

A geometry plugin keeps its constructor arguments and writes them into the
geometry slots of a component descriptor (``fill``).  The intersection code
itself runs inside the CUDA component kernels."""


class GPrim:
    kind = None

    def fill(self, comp, keep):
        """Write geometry kind and parameters into ``comp`` (a RampComp)."""
        comp.geom = self.kind

    def intersect_prg(self, *args, **kwargs):
        raise NotImplementedError(
            "geometry kernels run fused with their component's scatter kernel; "
            "use Instrument.execute")

    def lines(self):
        return [[0], [0], [0]]
