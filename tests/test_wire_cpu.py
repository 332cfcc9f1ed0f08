"""Host side of the wire format (no GPU): the C ABI's SHA-256 against
hashlib, message ids and slot layout against the restatement of
hmpc-rs/src/net/queue.rs and net.rs."""
import hashlib
import os
import random

import pytest

from hmpc_gb300 import _lib, wire
from oracle import wire_oracle


@pytest.mark.parametrize("size", [0, 1, 3, 55, 56, 63, 64, 65, 119, 128, 1000, 4097])
def test_sha256_matches_hashlib(size):
    data = random.Random(size).randbytes(size)
    assert wire.sha256(data) == hashlib.sha256(data).digest()


def test_sha256_known_answers():
    # FIPS 180-4 examples
    assert wire.sha256(b"abc").hex() == "ba7816bf8f01cfea414140de5dae2223b00361a396177a9cb410ff61f20015ad"
    assert wire.sha256(b"").hex() == "e3b0c44298fc1c149afbf4c8996fb92427ae41e4649b934ca495991b7852b855"


@pytest.mark.parametrize("kind,member", [(wire.BROADCAST, 0), (wire.BROADCAST, 2), (wire.GATHER, 1),
                                         (wire.ALL_GATHER, None), (wire.ALL_TO_ALL, None)])
@pytest.mark.parametrize("parties", [[0, 1, 2], [2, 0, 1, 1], [7], [65535, 3, 300]])
def test_message_ids_match_restatement(kind, member, parties):
    for counter in (1, 2, 1000):
        got = wire.message_id(kind, wire.U32, member, parties, parties, counter)
        assert got == wire_oracle.message_id(kind, wire.U32, member, parties, parties, counter)
    # senders and receivers enter separately (queue.rs:130-134)
    assert (wire.message_id(kind, wire.U32, member, parties, [9], 1) ==
            wire_oracle.message_id(kind, wire.U32, member, parties, [9], 1))


def test_layout_matches_restatement():
    sizes = [0, 1, 15, 16, 17, 1 << 20, 36]
    for flags in (0, wire.SESSIONS):
        offsets, total = wire.layout([{}] * len(sizes), sizes, flags)
        ref_offsets, ref_total = wire_oracle.layout(sizes, flags)
        assert offsets == ref_offsets and total == ref_total


def test_invalid_arguments_are_status_codes():
    lib = _lib.load()
    out = (_lib.ctypes.c_uint64 * 1)()
    assert lib.hmpc_wire_message_id(2, 0x21, None, 1, None, 0, None, 0, 1, out) == 1
    assert lib.hmpc_wire_layout(None, 0, 0, None, None) == 1
