"""pytest plugin: install this engine as gpufsm's CUDA backend before collection.

    pytest -p abstraction_regret_gb300.pytest_install <the reference's GPU test files>

runs the reference's own GPU tests, unchanged, against this engine: ``plugin.install()``
registers every technique into gpufsm's registry (src/gpufsm/core/registry.py:62-104)
and replaces its CUDA availability probe, so the tests' ``available_backends()`` and
``list_techniques(Backend.CUDA, ...)`` see this engine.
"""

from __future__ import annotations


def pytest_configure(config):  # noqa: ARG001 - pytest hook signature
    import gpufsm  # noqa: F401 - imports gpufsm.backends (its CUDA probe) first

    from . import plugin

    plugin.install()
