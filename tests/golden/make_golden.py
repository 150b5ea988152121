"""Writes tests/golden/scone_golden.json, the fixtures that pin the CPU oracle to SCONE.

Contents
  rng.*        draws and skip-ahead states of SCONE's 63-bit LCG (RandomNumbers/RNG_class.f90:40-44,
               147-168, 251-304) evaluated with Python integers, independent of the C++ code;
  pow_of_gsq   the 63-entry table of RandomNumbers/RNG_class.f90:61-123, parsed from the file;
  mgMat1/2     the 4-group data of IntegrationTestFiles/mgMat1 and mgMat2 (used by
               NuclearData/mgNeutronData/baseMgNeutron/Tests/baseMgNeutronDatabase_iTest.f90);
  h1_ace       the ESZ block (energy grid, total, absorption, elastic) and AW/TZ of the 1001.03c
               table in IntegrationTestFiles/1001JEF311.ace, the H-1 data that
               NuclearData/ceNeutronData/aceDatabase/Tests/aceNeutronDatabase_iTest.f90 reads.

Beside the JSON it writes tests/golden/scone_h1_1001_03c.ace: that 1001.03c table as it stands in
the file (header, NXS/JXS and its XSS lines, 12 + ceil(NXS(1)/4) lines from the line testLib
gives), so the tests read SCONE's own H-1 table without the SCONE tree.

Run from the repository root with $SCONE_REF naming a SCONE source tree; the committed files are
what the tests read, so the sources are only needed to regenerate them.  Without $SCONE_REF the
fields taken from SCONE are carried over from the committed JSON.
"""
import json
import os
import re

REF = os.environ.get("SCONE_REF", "")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "scone_golden.json")
H1_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "scone_h1_1001_03c.ace")

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


def parse_ace_esz(path, first_line):
    """ESZ block of the ACE table starting at 1-based line `first_line` (aceCard_class.f90:262-301):
    header line (ZAID AW TZ date), comment, 4 lines of IZ/AW pairs, NXS(16), JXS(32), then XSS."""
    lines = open(path).read().splitlines()[first_line - 1:]
    zaid, aw, tz = lines[0].split()[:3]
    ints = " ".join(lines[6:12]).split()
    nxs = [int(x) for x in ints[:16]]
    jxs = [int(x) for x in ints[16:48]]
    nes = nxs[2]
    need = jxs[0] - 1 + 4 * nes
    xss = []
    for ln in lines[12:]:
        xss.extend(float(x) for x in ln.split())
        if len(xss) >= need:
            break
    p = jxs[0] - 1
    blk = lambda k: xss[p + k * nes: p + (k + 1) * nes]
    return dict(zaid=zaid, aw=float(aw), tz=float(tz), e=blk(0), total=blk(1), absorption=blk(2),
                elastic=blk(3))


def ace_table_lines(path, first_line):
    """The lines of the ACE type-1 table that starts at 1-based line `first_line`: the header (2
    lines), IZ/AW (4), NXS and JXS (6), then NXS(1) XSS values four to a line."""
    lines = open(path).read().splitlines(keepends=True)[first_line - 1:]
    nxs1 = int(" ".join(lines[6:12]).split()[0])
    return lines[:12 + (nxs1 + 3) // 4]


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
    if REF and os.path.exists(tbl):
        gold["pow_of_gsq"] = [str(v) for v in parse_table(tbl)]
        gold["mgMat1"] = parse_mg(os.path.join(REF, "IntegrationTestFiles", "mgMat1"))
        gold["mgMat2"] = parse_mg(os.path.join(REF, "IntegrationTestFiles", "mgMat2"))
        lib = open(os.path.join(REF, "IntegrationTestFiles", "testLib")).read()
        line = int(re.search(r"1001\.03c;\s*(\d+);", lib).group(1))
        gold["h1_ace"] = parse_ace_esz(os.path.join(REF, "IntegrationTestFiles", "1001JEF311.ace"), line)
        with open(H1_OUT, "w") as f:
            f.writelines(ace_table_lines(os.path.join(REF, "IntegrationTestFiles", "1001JEF311.ace"), line))
        print("wrote", H1_OUT)
    elif os.path.exists(OUT):
        old = json.load(open(OUT))
        for k in ("pow_of_gsq", "mgMat1", "mgMat2", "h1_ace"):
            gold[k] = old[k]
    with open(OUT, "w") as f:
        json.dump(gold, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
