"""GB300-native CUDA backend for TransiFlow's finite-volume hot path.

    from transiflow_gb300 import Interface, Continuation
    interface = Interface({'Reynolds Number': 0}, 256, 256)
    continuation = Continuation(interface, newton_tolerance=1e-8)
    x0 = continuation.newton(interface.vector())
    x, mu = continuation.continuation(x0, 'Reynolds Number', 0, 5000, 200)

``Interface`` is a drop-in for ``transiflow.interface.SciPy.Interface`` and
``Continuation`` / ``TimeIntegration`` follow ``transiflow.Continuation`` /
``transiflow.TimeIntegration``; the reference's own drivers also run on the
interface unchanged.
"""

from .continuation import Continuation, TimeIntegration
from .interface import Interface, create
from .vector import DeviceVector

__all__ = ['Interface', 'create', 'Continuation', 'TimeIntegration', 'DeviceVector']
