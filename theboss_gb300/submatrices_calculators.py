"""Drop-in GB300 replacements for theboss's all-minors ("submatrices") permanent
calculators, the C&C-B ingredient:

  BSSubmatricesPermanentCalculatorInterface  bs_submatrices_permanent_calculator_interface.py:12-50
  BSSubmatricesPermanentCalculatorBase       bs_submatrices_permanent_calculator_base.py:17-65
  BSCCRyserSubmatricesPermanentCalculator    bs_cc_ryser_submatrices_permanent_calculator.py:16-119
  BSCCCHSubmatricesPermanentCalculator       bs_cc_ch_submatrices_permanent_calculator.py:25-105

``compute_permanents()`` returns a list of numpy.complex128 of length
len(input_state): entry i is perm(U[T, S - e_i]) (0 where S_i = 0), computed in
one GPU sweep; the one-particle edge case returns the input occupations
(bs_submatrices_permanent_calculator_base.py:157-158).
"""
from __future__ import annotations

import abc
from typing import List, Optional, Sequence

import numpy as np
from numpy import complex128

from . import _native


class BSSubmatricesPermanentCalculatorInterface(abc.ABC):
    @abc.abstractmethod
    def compute_permanents(self) -> List[complex128]:
        raise NotImplementedError

    @property
    @abc.abstractmethod
    def matrix(self):
        raise NotImplementedError

    @matrix.setter
    @abc.abstractmethod
    def matrix(self, matrix) -> None:
        raise NotImplementedError

    @property
    @abc.abstractmethod
    def input_state(self):
        raise NotImplementedError

    @input_state.setter
    @abc.abstractmethod
    def input_state(self, input_state) -> None:
        raise NotImplementedError

    @property
    @abc.abstractmethod
    def output_state(self):
        raise NotImplementedError

    @output_state.setter
    @abc.abstractmethod
    def output_state(self, output_state) -> None:
        raise NotImplementedError


class BSSubmatricesPermanentCalculatorBase(BSSubmatricesPermanentCalculatorInterface, abc.ABC):
    def __init__(self, matrix: Sequence[Sequence[complex]], input_state: Optional[Sequence[int]] = None,
                 output_state: Optional[Sequence[int]] = None) -> None:
        if output_state is None:
            output_state = []
        if input_state is None:
            input_state = []
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


class _GB300SubmatricesCalculator(BSSubmatricesPermanentCalculatorBase):
    _VARIANT = _native.RYSER

    def compute_permanents(self) -> List[complex128]:
        n = len(self._input_state)
        if len(self._output_state) != n:
            raise AttributeError
        U = _native.as_matrix(self._matrix)
        S = _native.as_states(self._input_state, n)
        T = _native.as_states(self._output_state, n)
        row = _native.submatrices_batch(U, S, T, self._VARIANT)[0]
        return [complex128(v) for v in row]


class BSCCRyserSubmatricesPermanentCalculator(_GB300SubmatricesCalculator):
    """One Ryser sweep over the input's Guan codes, products over the output's
    occupied modes with powers (bs_cc_ryser_submatrices_permanent_calculator.py:73-119)."""

    _VARIANT = _native.RYSER


class BSCCCHSubmatricesPermanentCalculator(_GB300SubmatricesCalculator):
    """Same minors as bs_cc_ch_submatrices_permanent_calculator.py:51-105."""

    _VARIANT = _native.CHIN_HUH


def _register_with_reference() -> None:
    try:
        from theboss.boson_sampling_utilities.permanent_calculators.bs_submatrices_permanent_calculator_interface import (
            BSSubmatricesPermanentCalculatorInterface as _Ref,
        )
    except Exception:
        return
    for cls in (BSCCRyserSubmatricesPermanentCalculator, BSCCCHSubmatricesPermanentCalculator):
        _Ref.register(cls)


_register_with_reference()
