"""InspireParams and InspireVariant (src/params.rs)."""
from __future__ import annotations

import enum
import math
from dataclasses import dataclass, field

from . import _native as nat

DEFAULT_CRT_MODULI = (268369921, 249561089)  # params.rs:31


class InspireVariant(enum.Enum):
    NoPacking = 0
    OnePacking = 1
    TwoPacking = 2


@dataclass
class InspireParams:
    """InspireParams (params.rs:135-185)."""

    ring_dim: int = 2048
    crt_moduli: tuple = DEFAULT_CRT_MODULI
    p: int = 1 << 16
    sigma: float = 6.4
    gadget_base: int = 1 << 20
    gadget_len: int = 3
    q: int = field(default=0)

    def __post_init__(self):
        self.crt_moduli = tuple(int(m) for m in self.crt_moduli)
        if not self.q:
            self.q = math.prod(self.crt_moduli)

    @classmethod
    def secure_128_d2048(cls, p: int = 65537) -> "InspireParams":
        """params.rs:213-230 (p = 65537 there; the benchmark configs use 2^16)."""
        q = math.prod(DEFAULT_CRT_MODULI)
        return cls(2048, DEFAULT_CRT_MODULI, p, 6.4, 1 << 20, math.ceil(math.log2(q) / 20), q)

    def delta(self) -> int:
        """Delta = floor(q / p) (params.rs:296-298)."""
        return self.q // self.p

    def moduli(self):
        return self.crt_moduli

    @property
    def crt_count(self) -> int:
        return len(self.crt_moduli)

    @property
    def plen(self) -> int:
        return self.ring_dim * self.crt_count

    def validate(self) -> None:
        """InspireParams::validate (params.rs:348-387)."""
        if self.ring_dim <= 0 or self.ring_dim & (self.ring_dim - 1):
            raise ValueError("ring_dim must be a power of two")
        if not self.crt_moduli:
            raise ValueError("crt_moduli must be non-empty")
        if len(self.crt_moduli) > 2:
            raise ValueError("crt_moduli length > 2 is not supported")
        for m in self.crt_moduli:
            if m % (2 * self.ring_dim) != 1:
                raise ValueError("CRT moduli must be ≡ 1 (mod 2d) for NTT")
        if self.q != math.prod(self.crt_moduli):
            raise ValueError("q must equal product of CRT moduli")
        if len(self.crt_moduli) == 2 and math.gcd(*self.crt_moduli) != 1:
            raise ValueError("CRT moduli must be coprime")
        if self.q < self.p:
            raise ValueError("q must be >= p")

    def to_c(self) -> nat.InspireParamsC:
        pc = nat.InspireParamsC()
        pc.ring_dim = self.ring_dim
        pc.crt_count = self.crt_count
        for i, m in enumerate(self.crt_moduli):
            pc.crt_moduli[i] = m
        pc.p = self.p
        pc.sigma = self.sigma
        pc.gadget_base = self.gadget_base
        pc.gadget_len = self.gadget_len
        return pc


def num_columns(entry_size: int) -> int:
    """ceil(entry_size * 8 / 16) 16-bit columns per entry (setup.rs:190-192)."""
    return max(1, (entry_size * 8 + 15) // 16)
