"""Extract the reference's own golden vectors into JSON fixtures.

The reference ships its known-answer data as generated C++ headers
(``tests/gen/random-tensors.hpp`` and ``tests/gen/random-tn.hpp``, produced by
``tests/gen/random-tensors-gen.py`` / ``random-tn-gen.py`` with numpy seed
9457). This script reads those headers as text and writes the same data as
JSON so that the test-suite can run without the reference checkout.

Usage::

    python tests/golden/make_golden.py /path/to/reference

Output: ``tests/golden/random_tensors.json`` and ``tests/golden/random_tn.json``.
Every complex number keeps the two-decimal text of the header (it is parsed
with ``float``), so the fixtures are exactly what the reference tests compare
against (``tests/c2-tensor.cpp:141-214``, ``tests/c2-mpi.cpp:80-214``,
``tests/c2-network.cpp:16-152``).
"""
import json
import os
import re
import sys

NUM = r"[+-]?\s*\d+\.\d+"
COMPLEX = re.compile(r"(" + NUM + r")\s*([+-]\s*\d+\.\d+)i")
INT_LIST = re.compile(r"\d+")


def _parse_complex_list(text):
    out = []
    for m in COMPLEX.finditer(text):
        re_part = float(m.group(1).replace(" ", ""))
        im_part = float(m.group(2).replace(" ", ""))
        out.append([re_part, im_part])
    return out


def _parse_tensor_info(body):
    """``{{ d0, d1 }, { e0, e1, ... }}`` -> dict(dims, els)."""
    m = re.match(r"\s*\{\{([^}]*)\},\s*\{([^}]*)\}\}", body)
    if not m:
        raise ValueError("cannot parse tensor_info: " + body[:80])
    dims = [int(x) for x in INT_LIST.findall(m.group(1))]
    els = _parse_complex_list(m.group(2))
    size = 1
    for d in dims:
        size *= d
    if len(els) != size:
        raise ValueError("element count %d != size %d" % (len(els), size))
    return {"dims": dims, "els": els}, body[m.end():]


def _parse_wires(text):
    pairs = re.findall(r"\{\s*(\d+)\s*,\s*(\d+)\s*\}", text)
    return [[int(a), int(b)] for a, b in pairs]


def parse_random_tensors(src):
    cases = {}
    for m in re.finditer(r"const contraction_validation (v\d+) \{(.*?)\n  \};", src, re.S):
        name, body = m.group(1), m.group(2)
        infos = []
        rest = body
        for _ in range(3):
            k = rest.index("tensor_info")
            info, rest = _parse_tensor_info(rest[k + len("tensor_info"):])
            infos.append(info)
        k = rest.index("std::vector<qtnh::wire>")
        wires = _parse_wires(rest[k + len("std::vector<qtnh::wire>"):])
        cases[name] = {"t1": infos[0], "t2": infos[1], "t3": infos[2], "wires": wires}
    groups = {}
    for m in re.finditer(r"const std::vector<contraction_validation> (\w+) \{([^}]*)\};", src):
        groups[m.group(1)] = [cases[v.strip()] for v in m.group(2).split(",")]
    return groups


def parse_random_tn(src):
    cases = {}
    for m in re.finditer(r"const tn_validation (v\d+) \{(.*?)\n  \};", src, re.S):
        name, body = m.group(1), m.group(2)
        k_t = body.index("std::vector<tensor_info>")
        k_b = body.index("std::vector<bond_info>")
        tensors_txt = body[k_t + len("std::vector<tensor_info>"):k_b]
        tensors = []
        rest = tensors_txt
        while "tensor_info" in rest:
            k = rest.index("tensor_info")
            info, rest = _parse_tensor_info(rest[k + len("tensor_info"):])
            tensors.append(info)
        bonds_and_result = body[k_b:]
        k_r = bonds_and_result.index("tensor_info")
        bonds_txt = bonds_and_result[:k_r]
        bonds = []
        for bm in re.finditer(r"bond_info \{\s*(\d+),\s*(\d+),\s*\{(.*)\}\}", bonds_txt):
            bonds.append({"t1": int(bm.group(1)), "t2": int(bm.group(2)), "wires": _parse_wires(bm.group(3))})
        result, _ = _parse_tensor_info(bonds_and_result[k_r + len("tensor_info"):])
        cases[name] = {"tensors": tensors, "bonds": bonds, "result": result}
    groups = {}
    for m in re.finditer(r"const std::vector<tn_validation> (\w+) \{([^}]*)\};", src):
        groups[m.group(1)] = [cases[v.strip()] for v in m.group(2).split(",")]
    return groups


def _tensor_tokens(info):
    out = [str(len(info["dims"]))] + [str(d) for d in info["dims"]] + [str(len(info["els"]))]
    for re_, im_ in info["els"]:
        out += [repr(re_), repr(im_)]
    return out


def write_text_fixtures(here, rt, tn):
    """Whitespace-separated copies of the fixtures for the C++ API test driver
    (tests/cpp/api_test.cpp): no JSON parser needed there."""
    with open(os.path.join(here, "random_tensors.txt"), "w") as f:
        for name, cases in rt.items():
            f.write("group %s %d\n" % (name, len(cases)))
            for c in cases:
                toks = _tensor_tokens(c["t1"]) + _tensor_tokens(c["t2"]) + _tensor_tokens(c["t3"])
                toks += [str(len(c["wires"]))] + [str(x) for w in c["wires"] for x in w]
                f.write(" ".join(toks) + "\n")
    with open(os.path.join(here, "random_tn.txt"), "w") as f:
        for name, cases in tn.items():
            f.write("group %s %d\n" % (name, len(cases)))
            for c in cases:
                toks = [str(len(c["tensors"]))]
                for t in c["tensors"]:
                    toks += _tensor_tokens(t)
                toks += [str(len(c["bonds"]))]
                for b in c["bonds"]:
                    toks += [str(b["t1"]), str(b["t2"]), str(len(b["wires"]))] + [str(x) for w in b["wires"] for x in w]
                toks += _tensor_tokens(c["result"])
                f.write(" ".join(toks) + "\n")


def main(argv):
    if len(argv) != 2:
        sys.exit("usage: make_golden.py <path of the reference checkout>")
    ref = argv[1]
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(ref, "tests", "gen", "random-tensors.hpp"), encoding="utf-8") as f:
        rt = parse_random_tensors(f.read())
    with open(os.path.join(ref, "tests", "gen", "random-tn.hpp"), encoding="utf-8") as f:
        tn = parse_random_tn(f.read())
    meta = {
        "source": "reference tests/gen/random-tensors.hpp (numpy seed 9457, two-decimal text)",
        "tolerance": {"single_contraction": 1e-5, "network": 1e-2},
    }
    with open(os.path.join(here, "random_tensors.json"), "w") as f:
        json.dump({"meta": meta, "groups": rt}, f, separators=(",", ":"))
    meta = dict(meta, source="reference tests/gen/random-tn.hpp (numpy seed 9457, two-decimal text)")
    with open(os.path.join(here, "random_tn.json"), "w") as f:
        json.dump({"meta": meta, "groups": tn}, f, separators=(",", ":"))
    write_text_fixtures(here, rt, tn)
    for k, v in rt.items():
        print("random_tensors", k, len(v))
    for k, v in tn.items():
        print("random_tn", k, len(v))


if __name__ == "__main__":
    main(sys.argv)
