"""Classical memory addresses for hybrid programs (quantumflow/cbits.py:15-80).

A :class:`Register` names a region of classical memory with a Quil data type;
indexing it gives an :class:`Addr`, the key under which a value lives in
``State.memory``.  Equality, hashing and ordering follow the reference so
that programs written against it address the same cells.
"""
from functools import total_ordering
from typing import Any, Hashable

__all__ = ["Register", "Addr"]

DTYPE = {"BIT", "REAL", "INT", "OCTET", "ANY"}

DEFAULT_REGION = "ro"


@total_ordering
class Register:
    """A named region of classical memory (quantumflow/cbits.py:24-50)."""

    def __init__(self, name: str = DEFAULT_REGION, dtype: str = "BIT") -> None:
        if dtype not in DTYPE:
            raise ValueError(f"unknown classical data type {dtype!r}")
        self.name = name
        self.dtype = dtype

    def __getitem__(self, key: Hashable) -> "Addr":
        return Addr(self, key)

    def _key(self):
        return (self.dtype, self.name)

    def __lt__(self, other: Any) -> bool:
        if not isinstance(other, Register):
            return NotImplemented
        return self._key() < other._key()

    def __eq__(self, other: Any) -> bool:
        if not isinstance(other, Register):
            return NotImplemented
        return self._key() == other._key()

    def __hash__(self) -> int:
        return hash(self._key())

    def __repr__(self) -> str:
        return f"Register({self.name!r}, {self.dtype!r})"


@total_ordering
class Addr:
    """One cell of a register (quantumflow/cbits.py:53-80)."""

    def __init__(self, register: Register, key: Hashable) -> None:
        self.register = register
        self.key = key

    @property
    def dtype(self) -> str:
        return self.register.dtype

    def __str__(self) -> str:
        return f"{self.register.name}[{self.key}]"

    def __repr__(self) -> str:
        return f"{self.register!r}[{self.key!r}]"

    def _key(self):
        return (self.register, self.key)

    def __lt__(self, other: Any) -> bool:
        if not isinstance(other, Addr):
            return NotImplemented
        return self._key() < other._key()

    def __eq__(self, other: Any) -> bool:
        if not isinstance(other, Addr):
            return NotImplemented
        return self._key() == other._key()

    def __hash__(self) -> int:
        return hash(self._key())
