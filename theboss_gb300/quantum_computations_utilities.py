"""Distances between distributions (quantum_computations_utilities.py:25-79 of
theboss), with theboss's summation order.

  count_total_variation_distance        half the l1 distance of two equally long
                                        probability lists (a sequential sum: numpy's
                                        cumsum runs in the same order as theboss's loop)
  count_total_variation_distance_dicts  the same for {outcome: probability} dicts,
                                        missing keys counting as 0
"""
from __future__ import annotations

from typing import Dict, List, Set, Tuple, Union

import numpy as np


def count_total_variation_distance(distribution1: Union[List[float], np.ndarray],
                                   distribution2: Union[List[float], np.ndarray]) -> float:
    assert len(distribution1) == len(distribution2), (
        f"Distributions must have equal lengths! Got: {len(distribution1)}and {len(distribution2)}!")
    if len(distribution1) == 0:
        return 0.0
    d = np.abs(np.asarray(distribution1, dtype=np.float64) - np.asarray(distribution2, dtype=np.float64))
    return float(np.cumsum(d)[-1] / 2)


def count_total_variation_distance_dicts(distribution_1: Dict[Tuple[int, ...], float],
                                         distribution_2: Dict[Tuple[int, ...], float]) -> float:
    keys: Set[Tuple[int, ...]] = set()
    keys.update(distribution_1.keys())
    keys.update(distribution_2.keys())
    # numpy's abs, as in theboss: the terms are numpy floats, which Python's sum adds
    # plainly (its compensated path is for exact floats only)
    return 0.5 * sum([np.abs(distribution_1.get(k, 0) - distribution_2.get(k, 0)) for k in keys])
