"""Install this engine as gpufsm's CUDA backend (the drop-in path).

    import gpufsm
    import abstraction_regret_gb300.plugin as plugin
    plugin.install()                       # registers every technique under Backend.CUDA
    gpufsm.run_batch(nfa, inputs, backend="cuda")            # -> this engine, default "auto"
    gpufsm.run_batch(dfa, inputs, backend="cuda", technique="gather")

``install`` uses only gpufsm's public extension point (src/gpufsm/core/registry.py:62-104:
``register``, ``register_availability``, ``set_unavailable_reason``). It registers each
technique name of this package for ``Kind.NFA`` / ``Kind.DFA`` with ``Backend.CUDA``,
declares ``auto`` / ``gather`` as defaults unless gpufsm already declared one (its own
``_cuda`` extension, when built, declares ``dense``, backends/cuda/nfa.py:136-137), and
replaces the CUDA availability probe with this library's (loaded + a device visible),
recording the reason when it says no. Executors receive gpufsm's own NFA/DFA objects
(the CSR and table layouts are the same) and return gpufsm's own ``Result`` objects, the
same objects as its ``batch_results`` builds (src/gpufsm/core/result.py:27-50: times on
result 0), so ``bench.oracle.require``, ``api.benchmark`` and the CLI see no difference.
They are built while the device runs and given their verdicts afterwards: gpufsm's
``batch_results`` builds each by keyword after the device has finished (about 1.5 ms for
2048 results, against 0.1 ms left after the launch here).
"""

from __future__ import annotations

from . import executors


class _Adapter:
    """Wrap an executor so it returns the host package's Result objects."""

    def __init__(self, inner, result_cls) -> None:
        self._inner = inner
        self._result_cls = result_cls

    def run(self, input_bytes: bytes):
        return self.run_batch([input_bytes])[0]

    def run_batch(self, inputs):
        return executors.run_batch_results(self._inner, list(inputs), self._result_cls)


def install(gpufsm_registry=None, gpufsm_result=None) -> list[str]:
    """Register this engine into gpufsm; returns the ``kind/technique`` names registered."""
    if gpufsm_registry is None:
        from gpufsm.core import registry as gpufsm_registry  # noqa: PLC0415
    if gpufsm_result is None:
        from gpufsm.core import result as gpufsm_result  # noqa: PLC0415
    R = gpufsm_registry
    Kind, Backend = R.Kind, R.Backend
    defaults = getattr(R, "_DEFAULTS", {})
    done = []

    def adapt(make):
        def factory(automaton, technique):
            return _Adapter(make(automaton, technique), gpufsm_result.Result)
        return factory

    for kind, names, make, default in (
            (Kind.NFA, executors.NFA_NAMES, executors.make_nfa_executor, "auto"),
            (Kind.DFA, executors.DFA_NAMES, executors.make_dfa_executor, "gather")):
        has_default = (kind, Backend.CUDA) in defaults
        for name in names:
            R.register(kind, Backend.CUDA, name,
                       default=(name == default and not has_default))(adapt(make))
            done.append(f"{kind.value}/{name}")

    def probe() -> bool:
        ok = executors.available()
        if not ok:
            from .registry import Backend as OurBackend, unavailable_reason

            R.set_unavailable_reason(Backend.CUDA, unavailable_reason(OurBackend.CUDA) or
                                     "libgbfsm unavailable")
        return ok

    R.register_availability(Backend.CUDA, probe)
    return done
