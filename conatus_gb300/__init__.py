"""conatus_gb300: the IMEX time-stepping hot path of conatus on one GB300 (sm_103a).

``install()`` routes the reference package's ``backend="cuda"`` (``Model.simulate``,
``Simulation``, ``IVPSolver``) to the device step of this package and, when no core is loaded,
inserts ``conatus_gb300.core`` as ``conatus._core`` (see ``conatus_gb300.reference_backend``).
"""


def install(precision: str = "fp64"):
    """Route the reference's ``backend="cuda"`` to the GB300 step; returns the reference package
    (``conatus_gb300.reference_backend.install``)."""
    from .reference_backend import install as _install
    return _install(precision)
