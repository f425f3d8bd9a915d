"""Fiat-Shamir transcript over the C-ABI state (src/transcript.rs).

The state is the POD ``z0p_transcript_state``; prove calls read it and leave
it exactly where the reference's ``&mut Transcript`` would be left.
"""
from __future__ import annotations

import ctypes as C

from ._lib import TranscriptState, check, lib


def _b(x) -> bytes:
    return x.encode() if isinstance(x, str) else bytes(x)


class Transcript:
    """Transcript::new(label) (src/transcript.rs:62-69)."""

    def __init__(self, label=b""):
        self.state = TranscriptState()
        lab = _b(label)
        check(lib().z0p_transcript_init(C.byref(self.state), lab, len(lab)))

    def clone(self) -> "Transcript":
        t = Transcript.__new__(Transcript)
        t.state = TranscriptState()
        C.memmove(C.byref(t.state), C.byref(self.state), C.sizeof(TranscriptState))
        return t

    def absorb(self, label, data) -> None:  # src/transcript.rs:72-77
        lab, d = _b(label), _b(data)
        check(lib().z0p_transcript_absorb(C.byref(self.state), lab, len(lab), d, len(d)))

    def challenge_bytes(self, label) -> bytes:
        lab = _b(label)
        out = (C.c_uint8 * 32)()
        check(lib().z0p_transcript_challenge_bytes(C.byref(self.state), lab, len(lab), out))
        return bytes(out)

    def challenge_ext(self, label):  # src/transcript.rs:136-141
        lab = _b(label)
        out = (C.c_uint32 * 4)()
        check(lib().z0p_transcript_challenge_ext(C.byref(self.state), lab, len(lab), out))
        return list(out)

    def challenge_index(self, label, domain: int):
        """Index below a power-of-two domain; None otherwise (src/transcript.rs:148-160)."""
        if domain <= 0 or domain & (domain - 1):
            return None
        lab = _b(label)
        out = C.c_uint64()
        check(lib().z0p_transcript_challenge_index(C.byref(self.state), lab, len(lab), domain,
                                                   C.byref(out)))
        return out.value

    def export(self) -> dict:
        s = self.state
        return {
            "tail": bytes(s.tail)[: s.tail_len],
            "stack": b"".join(bytes(s.stack[i]) for i in range(s.stack_len)),
            "stack_len": s.stack_len,
            "next_index": s.next_index,
            "total_len": s.total_len,
            "counter": s.counter,
        }
