"""Restatement of hmpc's network message format -- TEST INFRASTRUCTURE ONLY
(the checker for hmpc_gb300's device-side packer; the product never imports
it).

Follows hmpc-rs/src/net.rs:205-400 (SendMessage::write_to, ReceiveMessage::
build_from), hmpc-rs/src/net/queue.rs:108-135 (message ids) and
hmpc-rs/src/net/metadata.rs:3-76 (what the id hashes).  The reference has no
test vectors for this format; these functions are checked against the
documented layout (docs/networking.md "Message Format") and hashlib's SHA-256.
"""
import hashlib
import struct

VERSION = 0
SESSIONS = 1
SIGNING = 2


def header(kind, datatype, sender, receiver, message_id, flags=0, session=b""):
    """version u8, flags u8, kind u8, datatype u8, sender u16, receiver u16,
    id u64 (little-endian), then the 16-byte session id with the sessions
    feature (net.rs:237-245)"""
    h = struct.pack("<BBBBHHQ", VERSION, flags, kind, datatype, sender, receiver, message_id)
    if flags & SESSIONS:
        assert len(session) == 16
        h += session
    return h


def message(kind, datatype, sender, receiver, message_id, payload, flags=0, session=b""):
    return header(kind, datatype, sender, receiver, message_id, flags, session) + bytes(payload)


def parse(buf, flags=0, session=b""):
    """ReceiveMessage::build_from (net.rs:278-340): fields and payload, or a
    ValueError naming the first field that does not match"""
    if len(buf) < 16:
        raise ValueError("too short")
    version, fl, kind, datatype, sender, receiver, message_id = struct.unpack_from("<BBBBHHQ", buf)
    if version != VERSION:
        raise ValueError("version")
    if fl != flags:
        raise ValueError("flags")
    rest = buf[16:]
    if flags & SESSIONS:
        if rest[:16] != session:
            raise ValueError("session")
        rest = rest[16:]
    return dict(kind=kind, datatype=datatype, sender=sender, receiver=receiver, id=message_id), bytes(rest)


def _communicator(parties):
    ps = sorted(set(parties))
    return struct.pack("<Q", len(ps)) + b"".join(struct.pack("<H", p) for p in ps)


def message_id(kind, datatype, member, senders, receivers, counter):
    """initial id = first 8 bytes (LE) of SHA-256(senders, kind, datatype,
    member, receivers); the n-th operation with that hash uses initial + n
    (queue.rs:108-135)"""
    h = hashlib.sha256()
    h.update(_communicator(senders))
    h.update(struct.pack("<BB", kind, datatype))
    if member is not None:
        h.update(struct.pack("<H", member))
    h.update(_communicator(receivers))
    return (struct.unpack_from("<Q", h.digest())[0] + counter) & 0xFFFFFFFFFFFFFFFF


def layout(payload_sizes, flags=0):
    """16-byte aligned slots of header + payload"""
    hb = 32 if flags & SESSIONS else 16
    offsets, at = [], 0
    for n in payload_sizes:
        offsets.append(at)
        at += (hb + n + 15) // 16 * 16
    return offsets, at
