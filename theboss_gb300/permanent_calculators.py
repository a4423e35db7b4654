"""Drop-in GB300 replacements for theboss's permanent calculators.

Same names, constructor, properties, return types and exceptions as the classes
in theboss.boson_sampling_utilities.permanent_calculators:

  BSPermanentCalculatorInterface   bs_permanent_calculator_interface.py:18-52
  BSPermanentCalculatorBase        bs_permanent_calculator_base.py:22-72
  RyserPermanentCalculator         ryser_permanent_calculator.py:19-64
  ChinHuhPermanentCalculator       chin_huh_permanent_calculator.py:18-59
  GlynnGrayPermanentCalculator     glynn_gray_permanent_calculator.py:27-84
  ClassicPermanentCalculator       classic_permanent_calculator.py:18-67
  PermanentCalculatorType /
  BSPermanentCalculatorFactory     bs_permanent_calculator_factory.py:29-115

Every ``compute_permanent`` runs on the GPU (libboss_gb300.so); nothing is
computed on the host.  The calculators keep the caller's matrix by reference,
like theboss does, and read its current contents on every call, so in-place
updates (``calc.matrix *= sqrt(eta)``) are always seen.  They hold no GPU
handles, so they deep-copy and pickle like the originals.
"""
from __future__ import annotations

import abc
import enum
from typing import Optional, Sequence

import numpy as np
from numpy import complex128

from . import _native


class BSPermanentCalculatorInterface(abc.ABC):
    """bs_permanent_calculator_interface.py:18-52."""

    @abc.abstractmethod
    def compute_permanent(self) -> complex:
        raise NotImplementedError

    @property
    @abc.abstractmethod
    def matrix(self) -> Sequence[Sequence[complex]]:
        raise NotImplementedError

    @matrix.setter
    @abc.abstractmethod
    def matrix(self, matrix: Sequence[Sequence[complex]]) -> None:
        raise NotImplementedError

    @property
    @abc.abstractmethod
    def input_state(self) -> Sequence[int]:
        raise NotImplementedError

    @input_state.setter
    @abc.abstractmethod
    def input_state(self, input_state: Sequence[int]) -> None:
        raise NotImplementedError

    @property
    @abc.abstractmethod
    def output_state(self) -> Sequence[int]:
        raise NotImplementedError

    @output_state.setter
    @abc.abstractmethod
    def output_state(self, output_state: Sequence[int]) -> None:
        raise NotImplementedError


class BSPermanentCalculatorBase(BSPermanentCalculatorInterface, abc.ABC):
    """bs_permanent_calculator_base.py:22-72: state holder and the size check."""

    def __init__(
        self,
        matrix: Sequence[Sequence[complex128]],
        input_state: Optional[Sequence[int]] = None,
        output_state: Optional[Sequence[int]] = None,
    ) -> None:
        if output_state is None:
            output_state = list()
        if input_state is None:
            input_state = list()
        self._matrix = matrix
        self._input_state = input_state
        self._output_state = output_state

    @property
    def matrix(self):
        return self._matrix

    @matrix.setter
    def matrix(self, matrix) -> None:
        self._matrix = matrix

    @property
    def input_state(self):
        return self._input_state

    @input_state.setter
    def input_state(self, input_state) -> None:
        self._input_state = input_state

    @property
    def output_state(self):
        return self._output_state

    @output_state.setter
    def output_state(self, output_state) -> None:
        self._output_state = output_state

    def _can_calculation_be_performed(self) -> bool:
        return (
            len(self._matrix) == len(self._matrix[0])
            and len(self._output_state) == len(self._input_state)
            and len(self._output_state) <= len(self._matrix[0])
        )


class _GB300PermanentCalculator(BSPermanentCalculatorBase):
    _VARIANT = _native.RYSER

    def compute_permanent(self) -> complex128:
        if not self._can_calculation_be_performed():
            raise AttributeError
        n = len(self._input_state)
        U = _native.as_matrix(self._matrix)
        S = _native.as_states(self._input_state, n)
        T = _native.as_states(self._output_state, n)
        return complex128(_native.perm_batch(U, S, T, self._VARIANT)[0])

    def compute_permanents_of_outputs(self, output_states) -> np.ndarray:
        """All permanents U[T_k, S] for a list of output states, in one GPU launch
        (the batched form of a loop of ``compute_permanent`` calls)."""
        n = len(self._input_state)
        U = _native.as_matrix(self._matrix)
        T = _native.as_states(output_states, n)
        S = np.ascontiguousarray(np.broadcast_to(_native.as_states(self._input_state, n), T.shape))
        return _native.perm_batch(U, S, T, self._VARIANT)


class RyserPermanentCalculator(_GB300PermanentCalculator):
    """Ryser's formula over Guan codes of the input multiplicities
    (ryser_permanent_calculator.py:45-64)."""

    _VARIANT = _native.RYSER


class ChinHuhPermanentCalculator(_GB300PermanentCalculator):
    """Chin-Huh (Glynn with multiplicities) over Guan codes of the input
    multiplicities (chin_huh_permanent_calculator.py:38-59)."""

    _VARIANT = _native.CHIN_HUH


class GlynnGrayPermanentCalculator(_GB300PermanentCalculator):
    """Glynn's formula (glynn_gray_permanent_calculator.py:41-84).  The GPU sweeps
    Gray/Guan codes of whichever side has fewer codes, with one row fixed, which
    is the same value with fewer terms."""

    _VARIANT = _native.GLYNN

    def compute_permanent(self) -> complex128:
        if len(self._input_state) != len(self._output_state):
            raise AttributeError
        return super().compute_permanent()


class ClassicPermanentCalculator(_GB300PermanentCalculator):
    """Same value and zero-particle rules as classic_permanent_calculator.py:27-39
    (brute-force expansion there; a Glynn sweep here)."""

    _VARIANT = _native.CLASSIC

    def compute_permanent(self) -> complex128:
        if len(self._input_state) != len(self._output_state):
            raise AttributeError
        return super().compute_permanent()


class PermanentCalculatorType(enum.IntEnum):
    """bs_permanent_calculator_factory.py:29-33."""

    CLASSIC = enum.auto()
    GLYNN = enum.auto()
    CHIN_HUH = enum.auto()
    RYSER = enum.auto()


class BSPermanentCalculatorFactory:
    """bs_permanent_calculator_factory.py:36-115 (default RYSER, unknown types
    fall back to CHIN_HUH)."""

    def __init__(self, matrix, input_state, output_state,
                 calculator_type: PermanentCalculatorType = PermanentCalculatorType.RYSER):
        self._matrix = matrix
        self._input_state = input_state
        self._output_state = output_state
        self._calculator_type = calculator_type
        self._calculator_mapping = {
            PermanentCalculatorType.CLASSIC: ClassicPermanentCalculator,
            PermanentCalculatorType.GLYNN: GlynnGrayPermanentCalculator,
            PermanentCalculatorType.CHIN_HUH: ChinHuhPermanentCalculator,
            PermanentCalculatorType.RYSER: RyserPermanentCalculator,
        }

    @property
    def matrix(self):
        return self._matrix

    @matrix.setter
    def matrix(self, new_matrix) -> None:
        self._matrix = new_matrix

    @property
    def input_state(self):
        return self._input_state

    @input_state.setter
    def input_state(self, new_input_state) -> None:
        self._input_state = new_input_state

    @property
    def output_state(self):
        return self._output_state

    @output_state.setter
    def output_state(self, new_output_state) -> None:
        self._output_state = new_output_state

    def generate_calculator(self) -> BSPermanentCalculatorInterface:
        cls = self._calculator_mapping.get(self._calculator_type, ChinHuhPermanentCalculator)
        return cls(matrix=self.matrix, input_state=self.input_state, output_state=self.output_state)


def _register_with_reference() -> None:
    """When theboss itself is importable, make its abstract interface recognise
    these classes (isinstance / issubclass checks in user code keep working)."""
    try:
        from theboss.boson_sampling_utilities.permanent_calculators.bs_permanent_calculator_interface import (
            BSPermanentCalculatorInterface as _Ref,
        )
    except Exception:
        return
    for cls in (RyserPermanentCalculator, ChinHuhPermanentCalculator, GlynnGrayPermanentCalculator,
                ClassicPermanentCalculator):
        _Ref.register(cls)


_register_with_reference()
