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


# --- the format as the reference states it (tests/golden/reference_kats.json
# "wire", extracted from hmpc-rs/src/net.rs, hmpc-rs/src/net/queue.rs,
# hmpc-rs/src/net/metadata.rs and docs/networking.md) ------------------------

def header_defines():
    import pathlib
    import re

    text = (pathlib.Path(__file__).resolve().parents[1] / "include" / "hmpc_gb300.h").read_text()
    return {m.group(1): int(m.group(2), 0) for m in re.finditer(r"#define (HMPC_WIRE_\w+) (0x[0-9a-fA-F]+|\d+)", text)}


def test_message_kinds_are_the_references(kats):
    w = kats["wire"]
    kinds = {k: v["value"] for k, v in w["kinds"].items()}
    assert kinds == {"Send": 1, "Broadcast": 2, "Scatter": 3, "Gather": 4, "AllGather": 5, "AllToAll": 6,
                     "ConsistencyCheckBroadcast": 18, "ConsistencyCheckAllGather": 21}
    # the documentation's list agrees with the source
    doc = {k.replace(" ", ""): v["value"] for k, v in w["doc_kinds"].items()}
    assert all(doc[k] == kinds[k] for k in ("Send", "Broadcast", "Scatter", "Gather", "AllGather", "AllToAll"))
    assert doc["checkBroadcast"] == kinds["ConsistencyCheckBroadcast"] == kinds["Broadcast"] | 0x10
    assert doc["checkAllGather"] == kinds["ConsistencyCheckAllGather"] == kinds["AllGather"] | 0x10
    # the library's names (Python and the C header)
    ours = {"Send": wire.SEND, "Broadcast": wire.BROADCAST, "Scatter": wire.SCATTER, "Gather": wire.GATHER,
            "AllGather": wire.ALL_GATHER, "AllToAll": wire.ALL_TO_ALL}
    assert all(ours[k] == kinds[k] for k in ours)
    defines = header_defines()
    assert [defines[f"HMPC_WIRE_{n}"] for n in ("SEND", "BROADCAST", "SCATTER", "GATHER", "ALL_GATHER",
                                               "ALL_TO_ALL")] == [1, 2, 3, 4, 5, 6]


def test_feature_flags_and_version_are_the_references(kats):
    w = kats["wire"]
    assert w["version"]["value"] == wire_oracle.VERSION == 0
    assert w["feature_flags"]["sessions"]["bit"] == wire.SESSIONS == header_defines()["HMPC_WIRE_FLAG_SESSIONS"]
    assert w["feature_flags"]["signing"]["bit"] == wire.SIGNING == header_defines()["HMPC_WIRE_FLAG_SIGNING"]
    assert w["session_id_bytes"]["value"] == 16


def test_datatype_tag_rule(kats):
    """bit width | endianness (0x01 little-endian): the documented examples,
    and this library's 32-bit little-endian limbs"""
    for t in kats["wire"]["datatype_tags"]:
        assert t["bits"] | t["endianness"] == t["tag"]
    assert wire.U32 == (32 | 0x01) == header_defines()["HMPC_WIRE_DATATYPE_U32"]


def documented_layout(kats, mode):
    """byte offset -> (field symbol, byte index within the field) from the
    documentation's diagram for `mode`, payload bytes excluded"""
    rows = kats["wire"]["diagrams"][mode]["rows"]
    layout, seen = {}, {}
    for row in rows:
        for j, sym in enumerate(row["symbols"]):
            if sym == "d":
                continue
            offset = row["bit_offset"] // 8 + j
            layout[offset] = (sym, seen.get(sym, 0))
            seen[sym] = seen.get(sym, 0) + 1
    return layout


def test_header_bytes_follow_the_documented_diagrams(kats):
    w = kats["wire"]
    widths = {f["symbol"]: f["bits"] // 8 for f in w["doc_fields"]}
    # the write order of the reference's sender matches the diagram's order
    order = [o["field"].split(".")[-1] for o in w["write_order"]]
    assert order == ["MESSAGE_FORMAT_VERSION", "MESSAGE_FEATURE_FLAGS", "kind", "datatype", "sender", "receiver",
                     "id", "session", "data"]
    assert w["types"]["PartyID"]["bits"] == 16 and w["types"]["MessageID"]["bits"] == 64
    values = {"v": 0, "k": 0x12, "t": 0x21, "s": 0xBEEF, "r": 0x0102, "m": 0x1122334455667788}
    session = bytes(range(0xA0, 0xB0))
    for mode, flags in (("no features enabled", 0), ("sessions feature enabled", wire.SESSIONS)):
        layout = documented_layout(kats, mode)
        hdr = wire_oracle.header(values["k"], values["t"], values["s"], values["r"], values["m"], flags, session)
        assert len(hdr) == len(layout) == max(layout) + 1
        got = {}
        for offset, (sym, index) in layout.items():
            got.setdefault(sym, [0] * widths[sym])[index] = hdr[offset]
        expect = dict(values, f=flags)
        for sym, data in got.items():
            if sym == "i":
                assert bytes(data) == session
            else:
                assert int.from_bytes(bytes(data), "little") == expect[sym], (mode, sym)


def reference_message_id(kats, kind_name, datatype, member, senders, receivers, counter):
    """the message id computed from the extracted recipe alone: SHA-256 over
    the parts in hash_order (a communicator as its size then its distinct
    parties ascending, little-endian), the metadata = kind, datatype and the
    kind's member; the first 8 bytes (LE) plus the counter, which starts at the
    extracted counter_start"""
    w = kats["wire"]
    party = w["types"]["PartyID"]["bits"] // 8
    length = {"u64": 8}[w["communicator_length"]["type"]]

    def communicator(parties):
        ps = sorted(set(parties))
        return len(ps).to_bytes(length, "little") + b"".join(p.to_bytes(party, "little") for p in ps)

    h = hashlib.sha256()
    for part in w["hash_order"]:
        if part["part"] == "senders":
            h.update(communicator(senders))
        elif part["part"] == "receivers":
            h.update(communicator(receivers))
        else:
            h.update(bytes([w["kinds"][kind_name]["value"], datatype]))
            if w["hash_members"][kind_name]["member"] is not None:
                h.update(member.to_bytes(party, "little"))
    base = int.from_bytes(h.digest()[:8], "little")
    return (base + counter) % (1 << 64)


@pytest.mark.parametrize("kind_name,kind,member", [("Broadcast", wire.BROADCAST, 0), ("Broadcast", wire.BROADCAST, 5),
                                                   ("Gather", wire.GATHER, 1), ("AllGather", wire.ALL_GATHER, None),
                                                   ("AllToAll", wire.ALL_TO_ALL, None)])
def test_message_ids_follow_the_reference_recipe(kats, kind_name, kind, member):
    assert (kats["wire"]["hash_members"]["Broadcast"]["member"], kats["wire"]["hash_members"]["Gather"]["member"]) == \
        ("sender", "receiver")
    start = kats["wire"]["counter_start"]["value"]
    for parties, others in (([0, 1, 2], [0, 1, 2]), ([5, 3, 3, 9], [1]), ([65535], [0, 65535])):
        for n in range(3):
            counter = start + n  # the n-th operation with this hash
            got = wire.message_id(kind, wire.U32, member, parties, others, counter)
            assert got == reference_message_id(kats, kind_name, wire.U32, member or 0, parties, others, counter)
