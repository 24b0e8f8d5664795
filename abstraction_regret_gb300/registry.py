"""Technique registry: the extension point (reference: ``src/gpufsm/core/registry.py:27-162``).

Same model as the reference: factories ``(automaton, technique) -> Executor`` keyed by
``(Kind, Backend, technique)``, one declared default per ``(Kind, Backend)`` (a second,
different default raises ``RuntimeError``), availability probes per backend with a
recorded reason when a probe says no, and the same ``KeyError`` messages from
``get_factory``.

This package registers only ``Backend.CUDA``: it *is* the CUDA backend. The other enum
members exist so callers written against gpufsm still parse; asking them for a
technique raises the reference's "has no ... technique" ``KeyError``.
"""

from __future__ import annotations

from collections.abc import Callable
from enum import Enum
from typing import Any, Protocol, runtime_checkable

from .result import Result


class Kind(str, Enum):
    """Which automaton model a technique simulates."""

    NFA = "nfa"
    DFA = "dfa"

    @classmethod
    def of(cls, automaton: Any) -> Kind:
        """NFA or DFA, decided from the object (ours or the reference's)."""
        if hasattr(automaton, "trans") and hasattr(automaton, "accept"):
            return cls.DFA
        if hasattr(automaton, "sym_row_ptr") and hasattr(automaton, "eps_row_ptr"):
            return cls.NFA
        raise TypeError(f"expected an NFA or a DFA, got {type(automaton).__name__}")


class Backend(str, Enum):
    CPU = "cpu"
    TRITON = "triton"
    CUDA = "cuda"
    WARP = "warp"


@runtime_checkable
class Executor(Protocol):
    def run(self, input_bytes: bytes) -> Result: ...


ExecutorFactory = Callable[[Any, str], Executor]

_REGISTRY: dict[tuple[Kind, Backend, str], ExecutorFactory] = {}
_AVAILABILITY: dict[Backend, Callable[[], bool]] = {}
_DEFAULTS: dict[tuple[Kind, Backend], str] = {}
_UNAVAILABLE: dict[Backend, str] = {}


def register(
    kind: Kind, backend: Backend, technique: str, default: bool = False
) -> Callable[[ExecutorFactory], ExecutorFactory]:
    """Decorator registering ``factory`` under ``(kind, backend, technique)``.

    Re-registering the same triple replaces the factory. ``default=True`` declares the
    technique used when a caller names none; declaring a different one for the same
    ``(kind, backend)`` raises ``RuntimeError``.
    """

    def deco(factory: ExecutorFactory) -> ExecutorFactory:
        key = (kind, backend)
        if default and _DEFAULTS.get(key, technique) != technique:
            raise RuntimeError(
                f"two defaults declared for {backend.value}/{kind.value}: "
                f"{_DEFAULTS[key]!r} and {technique!r}"
            )
        _REGISTRY[(kind, backend, technique)] = factory
        if default:
            _DEFAULTS[key] = technique
        return factory

    return deco


def register_availability(backend: Backend, probe: Callable[[], bool]) -> None:
    _AVAILABILITY[backend] = probe


def set_unavailable_reason(backend: Backend, reason: str) -> None:
    """Record why ``backend``'s probe said no (shown by ``unavailable_reason``)."""
    _UNAVAILABLE[backend] = reason


def unavailable_reason(backend: Backend) -> str | None:
    return _UNAVAILABLE.get(backend)


def is_available(backend: Backend) -> bool:
    probe = _AVAILABILITY.get(backend)
    if probe is None:
        return any(b == backend for _, b, _ in _REGISTRY)
    try:
        return bool(probe())
    except Exception:
        return False


def list_techniques(backend: Backend, kind: Kind = Kind.NFA) -> list[str]:
    return [t for (k, b, t) in _REGISTRY if b == backend and k == kind]


def list_kinds(backend: Backend) -> list[Kind]:
    return [k for k in Kind if list_techniques(backend, k)]


def available_backends() -> list[Backend]:
    return [b for b in Backend if list_kinds(b) and is_available(b)]


def get_factory(kind: Kind, backend: Backend, technique: str | None) -> tuple[str, ExecutorFactory]:
    """Resolve ``technique`` (or the declared default when ``None``) to its factory."""
    techs = list_techniques(backend, kind)
    if not techs:
        why = (
            "the backend is not available on this machine (import or build failed)"
            if not is_available(backend)
            else f"it registers no {kind.value} technique"
        )
        raise KeyError(
            f"backend {backend.value!r} has no {kind.value} technique: {why}. "
            f"Available backends: {[b.value for b in available_backends()]}"
        )
    if technique is None:
        technique = _DEFAULTS.get((kind, backend))
        if technique is None:
            raise KeyError(
                f"backend {backend.value!r} declares no default {kind.value} technique; "
                f"name one explicitly (available: {techs}) or mark one with "
                f"register(..., default=True)"
            )
    factory = _REGISTRY.get((kind, backend, technique))
    if factory is None:
        raise KeyError(
            f"{kind.value} technique {technique!r} not registered for backend "
            f"{backend.value!r}; available: {techs}"
        )
    return technique, factory
