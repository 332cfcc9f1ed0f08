"""Messages of hmpc's network layer packed and unpacked on the device
(hmpc-rs/src/net.rs:205-400, docs/networking.md "Message Format"): one
message per (operation, receiver), the payload a tensor's limb-planar bytes."""
import ctypes

import torch

from . import _lib

SEND, BROADCAST, SCATTER, GATHER, ALL_GATHER, ALL_TO_ALL = 1, 2, 3, 4, 5, 6
SESSIONS, SIGNING = 1, 2
U32 = 0x21  # 32-bit little-endian limbs


def message_id(kind, datatype, member, senders, receivers, counter):
    """id of the `counter`-th operation (from 1) with this metadata"""
    mem = (ctypes.c_uint16 * 1)(member if member is not None else 0)
    s = (ctypes.c_uint16 * max(1, len(senders)))(*senders)
    r = (ctypes.c_uint16 * max(1, len(receivers)))(*receivers)
    out = ctypes.c_uint64()
    _lib.call("hmpc_wire_message_id", kind, datatype, mem, 0 if member is None else 1, s, len(senders), r,
              len(receivers), counter, ctypes.byref(out))
    return out.value


def sha256(data):
    digest = ctypes.create_string_buffer(32)
    _lib.call("hmpc_wire_sha256", bytes(data), len(data), digest)
    return digest.raw


def polynomial(tensor, i):
    """payload spec of polynomial i of a limb-planar batch Tensor: its L limb
    planes of N words (the storage of that polynomial as a tensor of its own)"""
    d = tensor.data
    return {"ptr": d.data_ptr() + 4 * i * tensor.n, "bytes": 4 * tensor.n * d.shape[0], "planes": d.shape[0],
            "plane_stride": 4 * d.shape[1]}


def _payload(t):
    if t is None:
        return None
    if isinstance(t, dict):
        return t
    return {"ptr": t.data_ptr(), "bytes": t.numel() * t.element_size(), "planes": 1, "plane_stride": 0}


def _messages(metas, payloads):
    arr = (_lib.WireMessage * len(metas))()
    for i, (m, t) in enumerate(zip(metas, payloads)):
        arr[i].kind = m["kind"]
        arr[i].datatype = m.get("datatype", U32)
        arr[i].sender = m["sender"]
        arr[i].receiver = m["receiver"]
        arr[i].id = m["id"]
        spec = _payload(t)
        if spec is not None:
            arr[i].payload = spec["ptr"]
            arr[i].bytes = spec["bytes"]
            arr[i].planes = spec["planes"]
            arr[i].plane_stride = spec["plane_stride"]
        else:
            arr[i].bytes = m["bytes"]
            arr[i].planes = m.get("planes", 1)
            arr[i].plane_stride = m.get("plane_stride", 0)
    return arr


def layout(metas, payload_bytes, flags=0):
    arr = (_lib.WireMessage * len(metas))()
    for i, n in enumerate(payload_bytes):
        arr[i].bytes = n
    offsets = (ctypes.c_uint64 * max(1, len(metas)))()
    total = ctypes.c_uint64()
    _lib.call("hmpc_wire_layout", arr, len(metas), flags, offsets, ctypes.byref(total))
    return list(offsets)[: len(metas)], total.value


def pack(queue, metas, tensors, flags=0, session=None):
    """one message per (meta, tensor) into a device byte buffer; returns
    (buffer, offsets, sizes)"""
    arr = _messages(metas, tensors)
    sizes_payload = [arr[i].bytes for i in range(len(metas))]
    offsets, total = layout(metas, sizes_payload, flags)
    out = torch.empty(total, dtype=torch.uint8, device=queue.device)
    offs = (ctypes.c_uint64 * max(1, len(metas)))(*offsets)
    _lib.call("hmpc_wire_pack", queue.handle, arr, len(metas), flags, session, offs, out.data_ptr())
    header = 32 if flags & SESSIONS else 16
    return out, offsets, [header + n for n in sizes_payload]


def unpack(queue, buf, offsets, sizes, metas, outputs, flags=0, session=None):
    """check each message against `metas` and copy the payloads into
    `outputs` (device tensors, or payload specs from `polynomial`); returns
    the status list (0 = ok, else the first mismatching field)"""
    count = len(metas)
    specs = [_payload(t) for t in outputs]
    arr = _messages(metas, specs)
    offs = (ctypes.c_uint64 * max(1, count))(*offsets)
    szs = (ctypes.c_uint64 * max(1, count))(*sizes)
    ptrs = (ctypes.c_void_p * max(1, count))(*[sp["ptr"] for sp in specs])
    status = torch.empty(count, dtype=torch.int32, device=queue.device)
    _lib.call("hmpc_wire_unpack", queue.handle, buf.data_ptr(), offs, szs, count, flags, session, arr, ptrs,
              status.data_ptr())
    return [int(v) for v in status.cpu().tolist()]
