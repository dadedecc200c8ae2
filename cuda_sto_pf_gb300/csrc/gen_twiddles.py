"""Generate rader41.cuh: constants of the radix-41 Rader stage.

    python cuda_sto_pf_gb300/csrc/gen_twiddles.py

A prime-length DFT of length p = 41 is rewritten (Rader 1968) as a cyclic
convolution of length 40 using the primitive root g = 6 (g^-1 = 7):
    X_0          = sum_n x_n
    X_{g^-q}     = x_0 + sum_{p'} x_{g^p'} W^{g^(p'-q)},   q = 0..39
                 = x_0 + (a (*) b)_q,  a_p = x_{g^p},  b_m = W^{g^-m}
The convolution is done as IFFT40(FFT40(a) . B) with B = FFT40(b) / 40
precomputed here (forward W = exp(-2 pi i / 41) and its conjugate for the
inverse transform), together with the FFT40 twiddles W40^e.
"""
import cmath
import os

P, G, GINV = 41, 6, 7
HERE = os.path.dirname(os.path.abspath(__file__))


def dft(x, sign=-1):
    n = len(x)
    return [sum(x[j] * cmath.exp(sign * 2j * cmath.pi * j * k / n) for j in range(n)) for k in range(n)]


def main():
    assert pow(G, 40, P) == 1 and all(pow(G, d, P) != 1 for d in (1, 2, 4, 5, 8, 10, 20))
    assert (G * GINV) % P == 1
    gpow = [pow(G, k, P) for k in range(40)]
    ginv = [pow(GINV, k, P) for k in range(40)]
    tables = {}
    for name, sign in (("fwd", -1), ("inv", +1)):
        w = cmath.exp(sign * 2j * cmath.pi / P)
        b = [w ** ginv[m] for m in range(40)]
        B = [v / 40.0 for v in dft(b, -1)]
        tables[name] = B
    w40 = [cmath.exp(-2j * cmath.pi * e / 40) for e in range(40)]
    # constexpr functions over local tables: usable in device code and
    # folded to immediates when the index is a compile-time constant
    lines = ["// Generated by gen_twiddles.py -- constants of the radix-41 Rader stage.",
             "#pragma once", "",
             "// a_p = x[rader41_gpow(p)] ; X[rader41_ginv(q)] = x_0 + c_q",
             "__host__ __device__ constexpr int rader41_gpow(int i) {",
             "    constexpr int t[40] = {" + ", ".join(map(str, gpow)) + "};",
             "    return t[i];", "}",
             "__host__ __device__ constexpr int rader41_ginv(int i) {",
             "    constexpr int t[40] = {" + ", ".join(map(str, ginv)) + "};",
             "    return t[i];", "}", ""]

    def arr(name, vals):
        body = ",\n        ".join(f"{v.real:.17e}, {v.imag:.17e}" for v in vals)
        return (f"__host__ __device__ constexpr double {name}(int i) {{\n"
                f"    constexpr double t[{2 * len(vals)}] = {{\n        {body}}};\n    return t[i];\n}}")

    lines.append("// B = FFT40(b) / 40, b_m = W41^{g^-m}; (re, im) pairs")
    lines.append(arr("rader41_bf", tables["fwd"]))
    lines.append(arr("rader41_bi", tables["inv"]))
    lines.append("// W40^e = exp(-2 pi i e / 40)")
    lines.append(arr("w40", w40))
    # cos / sin (2 pi i / 41): constants of the direct symmetric 41-point DFT
    lines.append("// cos(2 pi i / 41), sin(2 pi i / 41), i = 0..40")
    # exactly symmetric: values for i <= 20, mirrored (cos even, sin odd)
    cs = [cmath.cos(2 * cmath.pi * min(i, P - i) / P).real for i in range(P)]
    sn = [(1 if i <= P // 2 else -1) * cmath.sin(2 * cmath.pi * min(i, P - i) / P).real for i in range(P)]
    lines.append("__host__ __device__ constexpr double dft41_cos(int i) {\n"
                 "    constexpr double t[41] = {" + ", ".join(f"{v:.17e}" for v in cs) + "};\n    return t[i];\n}")
    lines.append("__host__ __device__ constexpr double dft41_sin(int i) {\n"
                 "    constexpr double t[41] = {" + ", ".join(f"{v:.17e}" for v in sn) + "};\n    return t[i];\n}")
    # the same B tables as __constant__ arrays for run-time (per-lane) indexing
    for prec, typ, mk in (("d", "double2", "make_double2"), ("f", "float2", "make_float2")):
        for key, nm in (("fwd", "BF"), ("inv", "BI")):
            body = ",\n    ".join(f"{{{v.real:.17e}, {v.imag:.17e}}}" for v in tables[key])
            lines.append(f"__constant__ {typ} c_rader41_{nm}_{prec}[40] = {{\n    {body}}};")
    with open(os.path.join(HERE, "rader41.cuh"), "w") as f:
        f.write("\n".join(lines) + "\n")
    # self-check of the construction in double precision
    import random
    x = [complex(random.random(), random.random()) for _ in range(P)]
    for sign, key in ((-1, "fwd"), (+1, "inv")):
        ref = dft(x, sign)
        a = [x[gpow[p]] for p in range(40)]
        A = dft(a, -1)
        C = [A[k] * tables[key][k] for k in range(40)]
        c = dft(C, +1)
        X = [0j] * P
        X[0] = sum(x)
        for q in range(40):
            X[ginv[q]] = x[0] + c[q]
        err = max(abs(X[k] - ref[k]) for k in range(P))
        assert err < 1e-11, err
    print("wrote rader41.cuh")


if __name__ == "__main__":
    main()
