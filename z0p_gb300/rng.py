"""ChaCha20 stream for masking randomness — mirrors z0p::rng::ChaCha20
(src/rng.rs:81-167). The state is the reference's fields, in order; a
zero-knowledge prove call advances it as the reference's prove_zk does."""
from __future__ import annotations

import ctypes as C

from ._lib import ChaChaState


class ChaCha20(ChaChaState):
    """ChaCha20::new(key, nonce) (src/rng.rs:101-112): counter 0, no buffered block."""

    @classmethod
    def new(cls, key: bytes, nonce: bytes) -> "ChaCha20":
        if len(key) != 32 or len(nonce) != 12:
            raise ValueError("key is 32 bytes, nonce 12 bytes")
        s = cls()
        C.memmove(s.key, key, 32)
        C.memmove(s.nonce, nonce, 12)
        s.counter = 0
        s.used = 64
        return s

    def export(self) -> dict:
        return {"key": bytes(self.key), "nonce": bytes(self.nonce), "counter": self.counter,
                "block": bytes(self.block), "used": self.used}
