"""Writes tests/golden/scone_golden.json, the fixtures that pin the CPU oracle to SCONE.

Contents
  rng.*        draws and skip-ahead states of SCONE's 63-bit LCG (RandomNumbers/RNG_class.f90:40-44,
               147-168, 251-304) evaluated with Python integers, independent of the C++ code;
  pow_of_gsq   the 63-entry table of RandomNumbers/RNG_class.f90:61-123, parsed from the file;
  mgMat1/2     the 4-group data of IntegrationTestFiles/mgMat1 and mgMat2 (used by
               NuclearData/mgNeutronData/baseMgNeutron/Tests/baseMgNeutronDatabase_iTest.f90).

Run from the repository root with the SCONE sources at $SCONE_REF (default /root/reference); the
committed JSON is what the tests read, so the sources are only needed to regenerate it.
"""
import json
import os
import re

REF = os.environ.get("SCONE_REF", "/root/reference")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "scone_golden.json")

G = 2806196910506780709
MASK = (1 << 63) - 1


def lcg_draws(seed, n):
    s = seed
    xs, states = [], []
    for _ in range(n):
        s = (G * s) & MASK
        s = (s + 1) & MASK
        states.append(s)
        xs.append(float(s) * 2.0 ** -63)
    return xs, states


def lcg_skip(seed, k):
    # direct affine power: s_k = g^k s + (g^k - 1)/(g - 1) mod 2^63, via repeated squaring
    k %= 1 << 63
    a, c = 1, 0          # accumulated map x -> a x + c
    ga, gc = G, 1        # map of one step
    while k:
        if k & 1:
            a, c = (ga * a) & MASK, (ga * c + gc) & MASK
        ga, gc = (ga * ga) & MASK, (ga * gc + gc) & MASK
        k >>= 1
    return (a * seed + c) & MASK


def parse_table(path):
    text = open(path).read()
    m = re.search(r"pow_of_gsq\s*=\s*\[(.*?)\]", text, re.S)
    return [int(x) for x in re.findall(r"(\d+)_int64", m.group(1))]


def parse_mg(path):
    text = re.sub(r"//[^\n]*", "", open(path).read())
    d = {}
    for key, body in re.findall(r"(\w+)\s*\(([^)]*)\)", text):
        d[key] = [float(x) for x in body.split()]
    d["numberOfGroups"] = int(re.search(r"numberOfGroups\s+(\d+)", text).group(1))
    return d


def main():
    seed = 0x5C3A84C9
    xs, st = lcg_draws(seed, 1000)
    skips = {str(k): lcg_skip(seed, k) for k in (1, 2, 152917, 13456757, 152917 * 1000000, (1 << 62) + 12345)}
    neg = {str(k): lcg_skip(seed, (1 << 63) + k) for k in (-1, -13456758)}
    gold = {
        "rng": {"seed": seed, "draws": xs[:64], "states": [str(s) for s in st[:64]], "state_1000": str(st[-1]),
                "skip": {k: str(v) for k, v in skips.items()}, "skip_negative": {k: str(v) for k, v in neg.items()}},
    }
    tbl = os.path.join(REF, "RandomNumbers", "RNG_class.f90")
    if os.path.exists(tbl):
        gold["pow_of_gsq"] = [str(v) for v in parse_table(tbl)]
        gold["mgMat1"] = parse_mg(os.path.join(REF, "IntegrationTestFiles", "mgMat1"))
        gold["mgMat2"] = parse_mg(os.path.join(REF, "IntegrationTestFiles", "mgMat2"))
    elif os.path.exists(OUT):
        old = json.load(open(OUT))
        for k in ("pow_of_gsq", "mgMat1", "mgMat2"):
            gold[k] = old[k]
    with open(OUT, "w") as f:
        json.dump(gold, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
