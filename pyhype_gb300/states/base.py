from __future__ import annotations

from typing import Union

import numpy as np


class RealizabilityException(Exception):
    pass


class State:
    """A (ny, nx, 4) float64 array plus the fluid it belongs to."""

    def __init__(self, fluid, state: "State" = None, array: np.ndarray = None,
                 shape: tuple = None, fill: Union[float, int] = None):
        self.fluid = fluid
        self._data = None
        if state is not None:
            self._data = np.zeros(state.shape)
            self.from_state(state)
        elif array is not None:
            self.data = array
        elif shape is not None:
            self.data = np.full(shape=shape, fill_value=fill if fill is not None else 0.0)
        else:
            raise ValueError("State constructor must recieve either a state, array or a shape.")

    @property
    def data(self) -> np.ndarray:
        return self._data

    @data.setter
    def data(self, array: np.ndarray) -> None:
        if not isinstance(array, np.ndarray):
            raise TypeError(f"Input array must be a Numpy array, but it is a {type(array)}.")
        if array.ndim != 3 or array.shape[-1] != 4:
            raise ValueError("Array must have 3 dims and a depth of 4.")
        if self._data is None or self._data.shape == array.shape:
            self._data = array
        else:
            self._data[:, :, :] = array

    @property
    def shape(self):
        return self._data.shape

    def make_non_dimensional(self) -> None:
        ff = self.fluid.far_field
        self._data[:, :, 0] /= ff.rho
        self._data[:, :, 1] /= ff.rho * ff.a
        self._data[:, :, 2] /= ff.rho * ff.a
        self._data[:, :, 3] /= ff.rho * ff.a ** 2

    def to_type(self, to_type):
        return to_type(fluid=self.fluid, array=_convert(self, to_type))

    def from_state(self, state: "State") -> None:
        if self.shape != state.shape:
            raise ValueError(f"States must have equal shape, but state has {self.shape} and from_state has {state.shape}")
        self.data = _convert(state, type(self))

    def realizable(self):
        conditions = self.realizability_conditions()
        if all(np.all(c) for c in conditions.values()):
            return True
        bad = {k: np.where(~v) for k, v in conditions.items() if not np.all(v)}
        return RealizabilityException(
            f"{self.__class__.__name__} has unrealizable values in the following conditions: {list(bad.values())}")

    def __getitem__(self, index) -> "State":
        return type(self)(fluid=self.fluid, array=self.data[index].copy())


def _convert(state: State, to_type) -> np.ndarray:
    from .conservative import ConservativeState
    from .primitive import PrimitiveState

    src = type(state)
    if issubclass(src, to_type) or src is to_type:
        return state.data.copy()
    if isinstance(state, ConservativeState) and issubclass(to_type, PrimitiveState):
        return np.dstack((state.rho.copy(), state.u, state.v, state.fluid.gm1() * (state.e - state.ek())))
    if isinstance(state, PrimitiveState) and issubclass(to_type, ConservativeState):
        return np.dstack((state.rho.copy(), state.rho * state.u, state.rho * state.v,
                          state.p / state.fluid.gm1() + state.ek()))
    raise TypeError(f"no conversion from {src.__name__} to {to_type.__name__}")
