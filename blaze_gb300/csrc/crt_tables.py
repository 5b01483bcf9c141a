"""Generate crt_tables.h: the reconstruction constants of the residue (CRT) product for every
modulus count N = 2..15.

The moduli are the first N of MODULI (pairwise coprime, at most 257, so that a residue in
[-128, 128] is exactly a BF16).  They are paired largest with smallest into super moduli
P_s = p q < 2^16 (N = 2 keeps both single, a modulus left over in the middle stays single), and a
super residue follows from the two residues c_p, c_q as

    u_s = (c_p A_s + c_q B_s) mod P_s,   A_s = (e_p y_s) mod P_s,  B_s = (e_q y_s) mod P_s,

with e_p = 1 mod p, 0 mod q (and e_q the other way round) and y_s = (P / P_s)^-1 mod P_s, so that
W = sum_s u_s (P / P_s) is congruent to the product modulo P = prod p.  Run: python crt_tables.py
"""
import os
import struct

MODULI = [257, 256, 255, 253, 251, 247, 241, 239, 233, 229, 227, 223, 217, 211, 199]
MAX_SUP = 8


def f32hex(x):
    """x rounded to FP32 (nearest), as an exact hexadecimal float literal."""
    return float(struct.unpack("<f", struct.pack("<f", x))[0]).hex()


def pairs(n):
    if n == 2:
        return [(0, -1), (1, -1)]
    out = [(t, n - 1 - t) for t in range(n // 2)]
    if n & 1:
        out.append((n // 2, -1))
    return out


def table(n):
    mods = MODULI[:n]
    P = 1
    for p in mods:
        P *= p
    sups = []
    for ia, ib in pairs(n):
        p = mods[ia]
        q = mods[ib] if ib >= 0 else 1
        sups.append(dict(ia=ia, ib=ib, p=p, q=q, Ps=p * q))
    for s in sups:
        Ps = s["Ps"]
        assert Ps < 1 << 16
        Ms = P // Ps
        ys = pow(Ms % Ps, -1, Ps)
        p, q = s["p"], s["q"]
        if q > 1:
            ep = q * pow(q, -1, p)  # 1 mod p, 0 mod q
            eq = p * pow(p, -1, q)  # 0 mod p, 1 mod q
            s["A"] = ep * ys % Ps
            s["B"] = eq * ys % Ps
        else:
            s["A"] = ys % Ps
            s["B"] = 0
        s["Psinv32"] = (1 << 32) // Ps
        s["pinv32"] = (1 << 32) // p
        s["qinv32"] = (1 << 32) // q if q > 1 else 0
        s["M"] = [(Ms >> (32 * l)) & 0xFFFFFFFF for l in range(4)]
        # the pair formula on every x < P_s, and its range before the reduction (32-bit Barrett)
        for x in range(Ps):
            cp, cq = x % p, x % q
            assert (cp * s["A"] + cq * s["B"]) % Ps == x * ys % Ps
        assert (p - 1) * s["A"] + (q - 1) * s["B"] < 1 << 26
    fbias = sum((1 << 23) / s["Ps"] for s in sups)
    limbs = (P.bit_length() + 1 + 31) // 32  # signed result |W| < P / 2
    return dict(n=n, P=P, sups=sups, fbias=fbias, limbs=limbs)


def emit(path):
    lines = [
        "// Generated by crt_tables.py: reconstruction constants of the residue product for N moduli.",
        "#pragma once",
        "#include <cstdint>",
        "",
        "namespace gb {",
        "",
        "struct CrtSuper {",
        "    int ia, ib;                 // residue planes (ib < 0: single modulus)",
        "    uint32_t p, q;              // q = 1 for a single modulus",
        "    uint32_t A, B;              // u = (c_p A + c_q B) mod P_s",
        "    uint32_t Ps, Psinv32;       // P_s and floor(2^32 / P_s)",
        "    uint32_t pinv32, qinv32;    // floor(2^32 / p), floor(2^32 / q)",
        "    uint32_t M[4];              // P / P_s, 32-bit limbs",
        "    float finv;                 // 1 / P_s rounded to FP32",
        "};",
        "",
        "struct CrtTable {",
        "    int nsup, limbs;            // super moduli; 32-bit limbs of the signed result",
        "    uint32_t P[4];              // product of the moduli, 32-bit limbs",
        "    float fbias;                // sum_s 2^23 / P_s rounded to FP32",
        f"    CrtSuper sup[{MAX_SUP}];",
        "};",
        "",
        "// index N - 2 for N = 2..15",
        "constexpr CrtTable kCrtTables[14] = {",
    ]
    for n in range(2, 16):
        t = table(n)
        P32 = ", ".join(f"{(t['P'] >> (32 * l)) & 0xFFFFFFFF}u" for l in range(4))
        lines.append(f"    {{{len(t['sups'])}, {t['limbs']}, {{{P32}}}, {f32hex(t['fbias'])}f, {{  // N = {n}")
        for s in t["sups"]:
            M = ", ".join(f"{m}u" for m in s["M"])
            finv = f32hex(1.0 / s["Ps"])
            lines.append(
                f"        {{{s['ia']}, {s['ib']}, {s['p']}u, {s['q']}u, {s['A']}u, {s['B']}u, {s['Ps']}u, "
                f"{s['Psinv32']}u, {s['pinv32']}u, {s['qinv32']}u, {{{M}}}, {finv}f}},"
            )
        lines.append("    }},")
    lines += ["};", "", "}  // namespace gb", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


if __name__ == "__main__":
    emit(os.path.join(os.path.dirname(os.path.abspath(__file__)), "crt_tables.h"))
