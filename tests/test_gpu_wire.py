"""Device-side packing of hmpc network messages against the restatement of
hmpc-rs/src/net.rs: the packed bytes, the round trip into fresh tensors, per
polynomial messages cut from a batch tensor, header checks and the
sessions feature."""
import numpy as np
import pytest
import torch

from hmpc_gb300 import _lib, lhe, wire
from hmpc_gb300.comp import Queue, Tensor
from oracle import wire_oracle

pytestmark = pytest.mark.gpu

Q_256 = 0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001
P_64 = 0x8822D80623320001
SESSION = bytes(range(16))


@pytest.fixture(scope="module")
def queue():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=[11] * 8)
    yield q
    q.close()


def meta(i, kind=wire.BROADCAST, sender=0, receiver=1):
    mid = wire_oracle.message_id(kind, wire.U32, sender, [0, 1, 2], [0, 1, 2], i + 1)
    return {"kind": kind, "sender": sender, "receiver": receiver, "id": mid}


@pytest.mark.parametrize("flags", [0, wire.SESSIONS])
def test_pack_matches_restatement_and_round_trips(queue, flags):
    gq = queue.modulus(Q_256)
    sizes = [(1,), (3,), (8,), (1,)]
    tensors = [queue.uniform(gq, s, 64 + 16 * i) for i, s in enumerate(sizes)]
    metas = [meta(i) for i in range(len(tensors))]
    session = SESSION if flags else None
    buf, offsets, msg_sizes = wire.pack(queue, metas, [t.data for t in tensors], flags, session)
    host = buf.cpu().numpy().tobytes()
    for t, m, off, size in zip(tensors, metas, offsets, msg_sizes):
        payload = t.data.cpu().numpy().tobytes()
        ref = wire_oracle.message(m["kind"], wire.U32, m["sender"], m["receiver"], m["id"], payload, flags,
                                  SESSION if flags else b"")
        assert host[off:off + size] == ref
        fields, body = wire_oracle.parse(host[off:off + size], flags, SESSION if flags else b"")
        assert fields["id"] == m["id"] and body == payload
    outs = [torch.empty_like(t.data) for t in tensors]
    metas_b = [dict(m, bytes=t.data.numel() * 4) for m, t in zip(metas, tensors)]
    status = wire.unpack(queue, buf, offsets, msg_sizes, metas_b, outs, flags, session)
    assert status == [0] * len(tensors)
    for t, o in zip(tensors, outs):
        assert torch.equal(t.data, o)


def test_per_ciphertext_messages_from_a_batch(queue):
    """each ciphertext of an encryption batch as its own message pair, cut
    from the batch tensors' limb planes, back into a fresh batch"""
    n, batch = 1 << 12, 6
    gq, gp = queue.modulus(Q_256), queue.modulus(P_64)
    s, key = lhe.keygen(queue, gq, gp, n)
    msgs = queue.uniform(gp, (batch,), n)
    ct = lhe.enc(queue, key, msgs, gq)
    metas, payloads = [], []
    for i in range(batch):
        for j, part in enumerate((ct.c0, ct.c1)):
            metas.append(meta(2 * i + j, kind=wire.SEND, receiver=2))
            payloads.append(wire.polynomial(part, i))
    buf, offsets, sizes = wire.pack(queue, metas, payloads)
    host = buf.cpu().numpy().tobytes()
    c0_host = ct.c0.numpy()
    body = wire_oracle.parse(host[offsets[2]:offsets[2] + sizes[2]])[1]  # ciphertext 1, c0
    assert body == np.ascontiguousarray(c0_host[:, n:2 * n]).tobytes()
    back = lhe.Ciphertext(Tensor(gq, (batch,), n), Tensor(gq, (batch,), n))
    back.c0.data.zero_()
    back.c1.data.zero_()
    outs = []
    for i in range(batch):
        outs += [wire.polynomial(back.c0, i), wire.polynomial(back.c1, i)]
    metas_b = [dict(m, bytes=p["bytes"], planes=p["planes"], plane_stride=p["plane_stride"])
               for m, p in zip(metas, payloads)]
    assert wire.unpack(queue, buf, offsets, sizes, metas_b, outs) == [0] * (2 * batch)
    assert torch.equal(back.c0.data, ct.c0.data) and torch.equal(back.c1.data, ct.c1.data)
    assert (lhe.dec(queue, s, back, gp).data == msgs.data).all().item()


def test_header_mismatches_are_reported_per_message(queue):
    gq = queue.modulus(Q_256)
    tensors = [queue.uniform(gq, (1,), 32) for _ in range(9)]
    metas = [meta(i) for i in range(9)]
    buf, offsets, sizes = wire.pack(queue, metas, [t.data for t in tensors], wire.SESSIONS, SESSION)
    expected = [dict(m, bytes=t.data.numel() * 4) for m, t in zip(metas, tensors)]
    # corrupt one field per message: version, flags, kind, datatype, sender, receiver, id, session
    for i, byte in enumerate([0, 1, 2, 3, 4, 6, 8, 16]):
        buf[offsets[i] + byte] ^= 0x40
    sizes = list(sizes)
    sizes[8] -= 4  # truncated
    outs = [torch.zeros_like(t.data) for t in tensors]
    status = wire.unpack(queue, buf, offsets, sizes, expected, outs, wire.SESSIONS, SESSION)
    assert status == [1, 2, 3, 4, 5, 6, 7, 8, 9]
    assert not any(o.any().item() for o in outs)  # nothing copied from a rejected message


def test_signing_feature_is_rejected(queue):
    gq = queue.modulus(Q_256)
    t = queue.uniform(gq, (1,), 32)
    with pytest.raises(_lib.HmpcError) as err:
        wire.pack(queue, [meta(0)], [t.data], wire.SIGNING)
    assert err.value.code == 2


@pytest.mark.parametrize("mode,flags", [("no features enabled", 0), ("sessions feature enabled", wire.SESSIONS)])
def test_device_headers_follow_the_documented_diagrams(queue, kats, mode, flags):
    """the packed header bytes read back at the offsets of the reference's
    own diagram (docs/networking.md "Visualizations", extracted into
    tests/golden/reference_kats.json), field widths from its field list, kinds
    and message ids from hmpc-rs (not from this repository's restatement)"""
    from test_wire_cpu import documented_layout, reference_message_id

    w = kats["wire"]
    widths = {f["symbol"]: f["bits"] // 8 for f in w["doc_fields"]}
    layout = documented_layout(kats, mode)
    gq = queue.modulus(Q_256)
    t = queue.uniform(gq, (2,), 64)
    kinds = [("Broadcast", 7, 3), ("Gather", 4, 9), ("AllToAll", 65535, 2)]
    metas = []
    for i, (name, sender, receiver) in enumerate(kinds):
        member = sender if name == "Broadcast" else receiver
        mid = reference_message_id(kats, name, wire.U32, member, [sender, receiver], [sender, receiver],
                                   w["counter_start"]["value"] + i)
        metas.append({"kind": w["kinds"][name]["value"], "sender": sender, "receiver": receiver, "id": mid})
    buf, offsets, sizes = wire.pack(queue, metas, [t.data] * len(metas), flags, SESSION if flags else None)
    host = buf.cpu().numpy().tobytes()
    payload = t.data.cpu().numpy().tobytes()
    for m, off, size in zip(metas, offsets, sizes):
        fields = {}
        for offset, (sym, index) in layout.items():
            fields.setdefault(sym, [0] * widths[sym])[index] = host[off + offset]
        value = {sym: int.from_bytes(bytes(b), "little") for sym, b in fields.items()}
        assert value["v"] == w["version"]["value"]
        assert value["f"] == flags
        assert (value["k"], value["t"], value["s"], value["r"], value["m"]) == \
            (m["kind"], wire.U32, m["sender"], m["receiver"], m["id"])
        if flags:
            assert bytes(fields["i"]) == SESSION
        header = max(layout) + 1
        assert host[off + header:off + size] == payload
