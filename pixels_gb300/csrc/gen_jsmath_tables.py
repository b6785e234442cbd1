"""Generate jsmath_tables.h: double-double constants for the correctly rounded
sin / atan2 of jsmath.cuh (values from mpmath at 200 bits).

Run: python pixels_gb300/csrc/gen_jsmath_tables.py > pixels_gb300/csrc/jsmath_tables.h
"""
import mpmath

mpmath.mp.prec = 200


def split(v, parts=2):
    out = []
    r = mpmath.mpf(v)
    for _ in range(parts):
        h = float(r)
        out.append(h)
        r -= mpmath.mpf(h)
    return out


def fmt(x):
    return float.hex(x)


lines = ["// Generated by gen_jsmath_tables.py (mpmath, 200-bit); do not edit.",
         "#pragma once", "",
         "// Each table exists twice: a __device__ copy for GPU code and a host copy;",
         "// PX_TAB(name) picks the one for the side being compiled.",
         "#if defined(__CUDACC__)",
         "#define PX_DEVTAB __device__ const",
         "#else",
         "#define PX_DEVTAB const",
         "#endif",
         "#if defined(__CUDA_ARCH__)",
         "#define PX_TAB(name) name##_d",
         "#else",
         "#define PX_TAB(name) name##_h",
         "#endif", ""]
pio2 = split(mpmath.pi / 2, 3)
lines.append("// pi/2 as three doubles (Cody-Waite reduction pieces)")
lines.append("#define PX_PIO2_1 %s\n#define PX_PIO2_2 %s\n#define PX_PIO2_3 %s" % tuple(fmt(v) for v in pio2))
pi = split(mpmath.pi, 2)
lines.append("#define PX_PI_HI %s\n#define PX_PI_LO %s" % tuple(fmt(v) for v in pi))
lines.append("#define PX_PIO2_HI %s\n#define PX_PIO2_LO %s" % tuple(fmt(v) for v in split(mpmath.pi / 2, 2)))
lines.append("#define PX_2OPI %s" % fmt(float(2 / mpmath.pi)))
lines.append("")
lines.append("// 1/n! for n = 0..30 as double-double (hi, lo)")
lines.append("static const double PX_INVFACT[31][2] = {")
for n in range(31):
    h, l = split(1 / mpmath.factorial(n))
    lines.append("  {%s, %s}," % (fmt(h), fmt(l)))
lines.append("};")
lines.append("")
lines.append("// atan(k/32) for k = 0..32 as double-double (hi, lo)")
lines.append("static const double PX_ATAN_TAB[33][2] = {")
for k in range(33):
    h, l = split(mpmath.atan(mpmath.mpf(k) / 32))
    lines.append("  {%s, %s}," % (fmt(h), fmt(l)))
lines.append("};")
lines.append("")
lines.append("// 1/(2n+1) for n = 0..15 as double-double (hi, lo)")
lines.append("static const double PX_INVODD[16][2] = {")
for n in range(16):
    h, l = split(mpmath.mpf(1) / (2 * n + 1))
    lines.append("  {%s, %s}," % (fmt(h), fmt(l)))
lines.append("};")
out = []
for ln in lines:
    if ln.startswith("static const double "):
        decl = ln[len("static const double "):]
        name, rest = decl.split("[", 1)
        out.append("__TABLE__%s|[%s" % (name, rest))
    else:
        out.append(ln)
# emit each table twice (device and host copies)
final = []
i = 0
while i < len(out):
    ln = out[i]
    if ln.startswith("__TABLE__"):
        name, rest = ln[len("__TABLE__"):].split("|", 1)
        body = []
        i += 1
        while out[i] != "};":
            body.append(out[i])
            i += 1
        for suffix, qual in (("_d", "static PX_DEVTAB double"), ("_h", "static const double")):
            final.append("%s %s%s%s" % (qual, name, suffix, rest))
            final.extend(body)
            final.append("};")
        i += 1
        continue
    final.append(ln)
    i += 1
print("\n".join(final))
