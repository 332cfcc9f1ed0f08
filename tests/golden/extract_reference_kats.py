"""Extract the known-answer vectors that pin hmpc's hot path from the
reference's own Catch2 test sources and write them to reference_kats.json.

The reference cannot be compiled in this environment (it needs a SYCL
compiler and C++23 deducing-this), so its tests are read as text: every value
in the JSON is copied from a REQUIRE/CHECK line or a literal in those files,
and each record carries the file:line it came from.

Usage (in a checkout that has the reference sources):
    python tests/golden/extract_reference_kats.py /path/to/hmpc
"""
import json
import pathlib
import re
import sys

HEX = r"0x[0-9a-fA-F']+"


def h(text):
    return int(text.replace("'", ""), 16)


def lines_of(path):
    return path.read_text().splitlines()


def chacha_vectors(root):
    rel = "tests/crypto/chacha.cpp"
    src = lines_of(root / rel)
    out = {"file": rel}

    # quarter round: inputs are declarations, outputs are REQUIREs
    qr_in, qr_out = {}, {}
    for no, line in enumerate(src, 1):
        m = re.search(r"hmpc::core::uint32 ([abcd]) = (" + HEX + r");", line)
        if m:
            qr_in[m.group(1)] = (h(m.group(2)), no)
        m = re.search(r"REQUIRE\(([abcd]) == (" + HEX + r")\);", line)
        if m:
            qr_out[m.group(1)] = (h(m.group(2)), no)
    out["quarter_round"] = {
        "input": [qr_in[k][0] for k in "abcd"],
        "output": [qr_out[k][0] for k in "abcd"],
        "lines": f"{rel}:{qr_in['a'][1]}-{qr_out['d'][1]}",
    }

    # block function and the additional vectors: replay the section as a tiny
    # program of array declarations, element assignments, chacha() calls and
    # REQUIREs on state words.
    arrays = {}
    blocks = []
    current = None
    pending_state = None
    calls = 0
    for no, line in enumerate(src, 1):
        m = re.search(r"hmpc::core::uint32 (?:const )?(key|nonce|counter)\[\] = \{([^}]*)\};", line)
        if m:
            arrays[m.group(1)] = [h(x.strip()) for x in m.group(2).split(",")]
            calls = 0
            continue
        m = re.search(r"\b(key|nonce|counter)\[(\d+)\] = (" + HEX + r");", line)
        if m:
            arrays[m.group(1)][int(m.group(2))] = h(m.group(3))
            continue
        if "chacha.param({key, nonce, counter});" in line:
            calls = 0
            continue
        if re.search(r"state = chacha\(\);", line):
            current = {
                "key": list(arrays["key"]),
                "nonce": list(arrays["nonce"]),
                "counter": arrays["counter"][0] + calls,
                "words": [None] * 16,
                "line": no,
            }
            calls += 1
            blocks.append(current)
            continue
        m = re.search(r"REQUIRE\(state\[(\d+)\] == (" + HEX + r")\);", line)
        if m and current is not None:
            current["words"][int(m.group(1))] = h(m.group(2))
            current["last_line"] = no
    for b in blocks:
        assert None not in b["words"], b
        b["lines"] = f"{rel}:{b.pop('line')}-{b.pop('last_line')}"
    out["blocks"] = blocks
    return out


def cipher_vectors(root):
    rel = "tests/crypto/cipher.cpp"
    text = (root / rel).read_text()

    def array(name):
        m = re.search(r"hmpc::core::uint(?:8|32) const " + name + r"\[\] =\s*\{([^}]*)\}", text)
        return [h(x.strip()) for x in m.group(1).replace("\n", " ").split(",") if x.strip()]

    start = text.index("plaintext_bytes[]")
    line = text[:start].count("\n") + 1
    return {
        "file": rel,
        "key": array("key"),
        "nonce": array("nonce"),
        "counter": array("counter")[0],
        "plaintext": array("plaintext_bytes"),
        "ciphertext": array("expected_ciphertext_bytes"),
        "lines": f"{rel}:{line}",
    }


def mod_vectors(root):
    rel = "tests/ints/mod.cpp"
    src = lines_of(root / rel)
    text = "\n".join(src)
    p = h(re.search(r"constexpr auto p = (" + HEX + r")_int;", text).group(1))
    out = {"file": rel, "p": p}
    for no, line in enumerate(src, 1):
        m = re.search(r"reduced_auxiliary_modulus == (" + HEX + r")_int", line)
        if m:
            out["R_mod_p"] = {"value": h(m.group(1)), "line": f"{rel}:{no}"}
        m = re.search(r"auto fivetwelve_montgomery = (" + HEX + r")_int;", line)
        if m:
            out["montgomery_512"] = {"value": h(m.group(1)), "line": f"{rel}:{no}"}
        m = re.search(r"mod_p\((-?)(" + HEX + r")_int\)\) == (" + HEX + r")_int", line)
        if m:
            out.setdefault("conversions", []).append({
                "input_negative": m.group(1) == "-",
                "input": h(m.group(2)),
                "canonical": h(m.group(3)),
                "line": f"{rel}:{no}",
            })
    return out


def poly_mod_vectors(root):
    rel = "tests/ints/poly_mod.cpp"
    src = lines_of(root / rel)
    text = "\n".join(src)
    p = h(re.search(r"constexpr auto p = (" + HEX + r")_int;", text).group(1))
    log_n = int(re.search(r"constexpr hmpc::size N = 1 << (\d+);", text).group(1))
    out = {"file": rel, "q": p, "N": 1 << log_n, "input": "x_i = i (canonical), every polynomial"}
    outputs = []
    for no, line in enumerate(src, 1):
        m = re.search(r"static_cast<integer>\(y\.root\) == (" + HEX + r")_int", line)
        if m:
            out["root"] = {"value": h(m.group(1)), "line": f"{rel}:{no}"}
        m = re.search(r"static_cast<integer>\(ntt_y\.root\) == (" + HEX + r")_int", line)
        if m:
            out["inverse_root"] = {"value": h(m.group(1)), "line": f"{rel}:{no}"}
        m = re.search(r"index_type\{j, (\d+)\}\]\)\) == (" + HEX + r")_int", line)
        if m:
            outputs.append({"index": int(m.group(1)), "canonical": h(m.group(2)), "line": f"{rel}:{no}"})
    out["ntt_outputs"] = outputs
    return out


def root_of_unity_vectors(root):
    rel = "tests/ints/num/theory/root_of_unity.cpp"
    text = (root / rel).read_text()
    p = int(re.search(r"constexpr auto p = 0b([01']+)_int;", text).group(1).replace("'", ""), 2)
    log_n = int(re.search(r"constexpr hmpc::size n = 1 << (\d+);", text).group(1))
    return {"file": rel, "p": p, "degree": 1 << log_n, "property": "root^degree == 1, root^i != 1 for 0 < i < degree"}


def lhe_vectors(root):
    rel = "tests/expr/crypto/lhe/enc.cpp"
    text = (root / rel).read_text()
    p = h(re.search(r"constexpr auto p = (" + HEX + r")_int;", text).group(1))
    q = h(re.search(r"constexpr auto q = (" + HEX + r")_int;", text).group(1))
    log_n = int(re.search(r"constexpr auto N = hmpc::size\{1\} << (\d+);", text).group(1))
    shape = [int(x) for x in re.search(r"auto shape = hmpc::shape\{(\d+), (\d+)\};", text).groups()]
    return {
        "file": rel,
        "p": p,
        "q": q,
        "N": 1 << log_n,
        "shape": shape,
        "key": "a = b = raw Montgomery representative i; s = Montgomery one",
        "plaintext": "NTT_p representation, raw representative i",
        "property": "dec(s, enc(key, x, randomness)) == x",
    }


def matvec_vectors(root):
    """tests/expr/matrix_vector_product.cpp: a matrix of bit monomials (an
    index tensor, std::nullopt for no monomial) times polynomials of degree
    N with small integer coefficients, and the signed products it CHECKs."""
    rel = "tests/expr/matrix_vector_product.cpp"
    src = lines_of(root / rel)
    text = "\n".join(src)
    log_n = int(re.search(r"constexpr hmpc::size N = 1 << (\d+);", text).group(1))
    rows = int(re.search(r"constexpr hmpc::size V = (\d+);", text).group(1))
    cols = {"four": 4, "two": 2, "eight": 8}[re.search(r"constexpr auto U = hmpc::constants::(\w+);", text).group(1)]
    index_shape = [int(x) if x.isdigit() else {"V": rows, "U": cols}[x]
                   for x in re.search(r"index_shape = hmpc::shape\{(\w+), (\w+), (\w+)\};", text).groups()]
    degrees, x, z = {}, {}, {}
    first = last = None
    for no, line in enumerate(src, 1):
        m = re.search(r"indices\[hmpc::index\{(\d+), (\d+), (\d+)\}\] = (\d+|std::nullopt);", line)
        if m:
            key = tuple(int(v) for v in m.groups()[:3])
            degrees[key] = -1 if m.group(4) == "std::nullopt" else int(m.group(4))
            first = first or no
        m = re.search(r"\bx\[hmpc::index\{(\d+), (\d+), (\d+)\}\] = uint\{(\d+)\};", line)
        if m:
            x[tuple(int(v) for v in m.groups()[:3])] = int(m.group(4))
        m = re.search(r"CHECK\(z\[hmpc::index\{(\d+), (\d+), (\d+)\}\] == (-?)integer\{(\d+)\}\);", line)
        if m:
            value = int(m.group(5))
            z[tuple(int(v) for v in m.groups()[:3])] = -value if m.group(4) else value
            last = no
    batch = index_shape[0]
    n = 1 << log_n
    return {
        "file": rel,
        "lines": f"{rel}:{first}-{last}",
        "n": n,
        "batch": batch,
        "rows": rows,
        "cols": cols,
        # degrees[b][i][k], -1 = std::nullopt
        "degrees": [[[degrees[(b, i, k)] for k in range(cols)] for i in range(rows)] for b in range(batch)],
        # x[b][k][c] and z[b][i][c]
        "x": [[[x[(b, k, c)] for c in range(n)] for k in range(cols)] for b in range(batch)],
        "z": [[[z[(b, i, c)] for c in range(n)] for i in range(rows)] for b in range(batch)],
    }


def reduce_vectors(root):
    """tests/expr/reduce.cpp: x_i = 3i + 1 and y_i = i + 1 as uint<127>, the
    reductions of x and the all/any of x == y that it CHECKs."""
    rel = "tests/expr/reduce.cpp"
    src = lines_of(root / rel)
    text = "\n".join(src)
    count = int(re.search(r"constexpr auto N = (\d+);", text).group(1))
    bits = int(re.search(r"using uint = hmpc::ints::uint<(\d+)>;", text).group(1))
    ax, bx = (int(v) for v in re.search(r"access_x\[i\] = uint\{static_cast<limb>\((\d+) \* i \+ (\d+)\)\};",
                                         text).groups())
    ay = re.search(r"access_y\[i\] = uint\{static_cast<limb>\(i \+ (\d+)\)\};", text)
    checks = {}
    names = {"sum": "add", "product": "multiply", "bit_or": "bit_or", "bit_and": "bit_and", "bit_xor": "bit_xor",
             "min": "min", "max": "max"}
    current = None
    for no, line in enumerate(src, 1):
        m = re.search(r"host_accessor (\w+)\((\w+)_tensor, hmpc::access::read\);", line)
        if m:
            current = m.group(1)
        m = re.search(r"CHECK\(value == uint\{(\d+)\}\);", line)
        if m and current in names:
            checks[names[current]] = {"value": int(m.group(1)), "line": f"{rel}:{no}"}
        m = re.search(r"size_limb_span<limb>\(([\d']+)\)\)\);", line)
        if m and current in names:
            checks[names[current]] = {"value": int(m.group(1).replace("'", "")), "line": f"{rel}:{no}"}
        m = re.search(r"CHECK(_FALSE)?\(value( == hmpc::bit\{true\})?\);", line)
        if m and current in ("all", "any"):
            key = {"all": "all_x_eq_y", "any": "any_x_eq_y"}[current]
            if current == "all" and "all_equal_tensor" in "\n".join(src[max(0, no - 4):no]):
                key = "all_x_eq_x"
            checks.setdefault(key, {"value": m.group(1) is None, "line": f"{rel}:{no}"})
    return {
        "file": rel,
        "count": count,
        "bits": bits,
        "x": [ax * i + bx for i in range(count)],
        "y": [i + int(ay.group(1)) for i in range(count)],
        "checks": checks,
    }


def wire_vectors(root):
    """hmpc's network message format as the reference states it: the
    message-kind tags, type widths, feature bits and write order of
    hmpc-rs/src/net.rs, the field list, byte diagrams, kind list and
    datatype-tag examples of docs/networking.md, the message-id counter of
    hmpc-rs/src/net/queue.rs and what the id hashes (hmpc-rs/src/net/metadata.rs)"""
    out = {}
    rel = "hmpc-rs/src/net.rs"
    src = lines_of(root / rel)
    kinds, in_enum = {}, False
    for no, line in enumerate(src, 1):
        if "pub enum MessageKind" in line:
            in_enum = True
        elif in_enum and line.strip() == "}":
            in_enum = False
        elif in_enum:
            m = re.match(r"\s*(\w+) = (\d+),", line)
            if m:
                kinds[m.group(1)] = {"value": int(m.group(2)), "line": f"{rel}:{no}"}
    out["kinds"] = kinds
    types = {}
    for no, line in enumerate(src, 1):
        m = re.match(r"pub type (\w+) = u(\d+);", line)
        if m:
            types[m.group(1)] = {"bits": int(m.group(2)), "line": f"{rel}:{no}"}
        m = re.match(r"const MESSAGE_FORMAT_VERSION: u8 = (\d+);", line)
        if m:
            out["version"] = {"value": int(m.group(1)), "line": f"{rel}:{no}"}
        m = re.match(r"const SESSION_ID_SIZE: usize = (\d+) / 8;", line)
        if m:
            out["session_id_bytes"] = {"value": int(m.group(1)) // 8, "line": f"{rel}:{no}"}
    out["types"] = types
    flags, names = {}, {}
    for no, line in enumerate(src, 1):
        m = re.search(r'let (\w+) = cfg!\(feature = "(\w+)"\) as u8;', line)
        if m:
            names[m.group(1)] = m.group(2)
        m = re.search(r"\| \((\w+) << (\d+)\)", line)
        if m and m.group(1) in names:
            flags[names[m.group(1)]] = {"bit": 1 << int(m.group(2)), "line": f"{rel}:{no}"}
        elif re.match(r"\s*(\w+)$", line.strip()) and line.strip() in names:
            flags[names[line.strip()]] = {"bit": 1, "line": f"{rel}:{no}"}
    out["feature_flags"] = flags
    order, in_write = [], False
    for no, line in enumerate(src, 1):
        if "async fn write_to(" in line:
            in_write = True
        elif in_write and "Ok(())" in line:
            break
        elif in_write:
            m = re.search(r"stream\.write_all\(([\w.]+?)(?:\.to_le_bytes\(\)\.as_slice\(\))?\)\.await", line)
            if m:
                order.append({"field": m.group(1), "line": f"{rel}:{no}"})
    out["write_order"] = order

    rel = "docs/networking.md"
    src = lines_of(root / rel)
    fields = []
    for no, line in enumerate(src, 1):
        m = re.search(r"\[([\w ]+)\]\(#[\w-]+\) \((\d+) bit, `(\w)`\)", line)
        if m:
            fields.append({"name": m.group(1), "bits": int(m.group(2)), "symbol": m.group(3), "line": f"{rel}:{no}"})
    out["doc_fields"] = fields
    diagrams, title = {}, None
    for no, line in enumerate(src, 1):
        t = line.strip()
        if t.endswith("enabled") and not t.startswith("-"):
            title = t
            diagrams[title] = {"rows": [], "line": f"{rel}:{no}"}
            continue
        m = re.match(r"\s*(\d+) \| ([a-z ]+) \|", line)
        if m and title:
            diagrams[title]["rows"].append({"bit_offset": int(m.group(1)), "symbols": m.group(2).split()})
    out["diagrams"] = diagrams
    doc_kinds = {}
    for no, line in enumerate(src, 1):
        m = re.match(r"- \[([\w ]+)\]\(#[\w-]+\) = (\d+)$", line.strip())
        if m:
            doc_kinds[m.group(1)] = {"value": int(m.group(2)), "line": f"{rel}:{no}"}
        m = re.match(r"- Check consistency of \[([\w ]+)\]\(#[\w-]+\) = (\d+)$", line.strip())
        if m:
            doc_kinds["check " + m.group(1)] = {"value": int(m.group(2)), "line": f"{rel}:{no}"}
    out["doc_kinds"] = doc_kinds
    tags = []
    for no, line in enumerate(src, 1):
        m = re.search(r"`0x([0-9a-f]{2}) \| 0x([0-9a-f]{2}) = 0x([0-9a-f]{2})`", line)
        if m:
            tags.append({"bits": int(m.group(1), 16), "endianness": int(m.group(2), 16), "tag": int(m.group(3), 16),
                         "line": f"{rel}:{no}"})
    out["datatype_tags"] = tags

    rel = "hmpc-rs/src/net/queue.rs"
    src = lines_of(root / rel)
    for no, line in enumerate(src, 1):
        if ".or_insert(" in line:
            out["counter_start"] = {"value": int(re.search(r"or_insert\((\d+)\)", line).group(1)),
                                    "line": f"{rel}:{no}"}
        if re.match(r"\s*id \+ counter\s*$", line):
            out["id_plus_counter"] = {"line": f"{rel}:{no}"}
        if "key.first_chunk::<MESSAGE_ID_SIZE>()" in line:
            out["id_from_hash_prefix"] = {"line": f"{rel}:{no}"}

    rel = "hmpc-rs/src/net/metadata.rs"
    src = lines_of(root / rel)
    hash_order, in_hash = [], False
    members = {}
    for no, line in enumerate(src, 1):
        if re.search(r"fn hash\(&self, senders", line):
            in_hash = True
        elif in_hash and "sha.finish()" in line:
            in_hash = False
        elif in_hash:
            m = re.search(r"(hash_communicator\((\w+)|hash_metadata)", line)
            if m:
                hash_order.append({"part": m.group(2) or "metadata", "line": f"{rel}:{no}"})
        m = re.match(r"message!\((\w+)(?:, (\w+))?\);", line)
        if m:
            members[m.group(1)] = {"member": m.group(2), "line": f"{rel}:{no}"}
        if "let len = communicator.len() as u64;" in line:
            out["communicator_length"] = {"type": "u64", "line": f"{rel}:{no}"}
    out["hash_order"] = hash_order
    out["hash_members"] = members
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: extract_reference_kats.py /path/to/hmpc")
    root = pathlib.Path(sys.argv[1])
    data = {
        "source": "hmpc v0.5.2 Catch2 tests, read as text",
        "chacha20": chacha_vectors(root),
        "cipher": cipher_vectors(root),
        "mod": mod_vectors(root),
        "poly_mod_ntt": poly_mod_vectors(root),
        "root_of_unity": root_of_unity_vectors(root),
        "linear_bgv": lhe_vectors(root),
        "matrix_vector_product": matvec_vectors(root),
        "reduce": reduce_vectors(root),
        "wire": wire_vectors(root),
    }
    out = pathlib.Path(__file__).with_name("reference_kats.json")
    out.write_text(json.dumps(data, indent=1, default=str) + "\n")
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
