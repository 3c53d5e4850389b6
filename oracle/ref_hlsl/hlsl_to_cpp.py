"""Mechanical HLSL -> C++ rewrite of the reference's compute shaders.

TEST INFRASTRUCTURE ONLY.  Reads the shader files where they lie in the
reference checkout (source/renderer/shaders/*.hlsl, *.hlsl.h and
wavefront/*.hlsl) and writes rewritten copies under an output folder that is
git-ignored (oracle/_ref/hlsl/); oracle/ref_hlsl/ref_trace.cpp and
ref_shade.cpp then include them together with oracle/ref_hlsl/hlsl_shim.h.

Every transform is syntactic and leaves the arithmetic, the control flow and
the order of operations of the shaders as written:

  1. `inout T name` parameters become `T& name` (HLSL copy-in/copy-out and a
     C++ reference agree for these non-aliased arguments).
  2. `(T)0` / `(T) 0` zero-initialisation casts become `T{}`.
  3. Register bindings (`: register(b0, space0)`) and system-value semantics
     (`: SV_DispatchThreadID`) are dropped.
  4. Attributes (`[numthreads(...)]`, `[branch]`, `[flatten]`, `[unroll]`,
     `[loop]`) are dropped.
  5. `Texture2D<float4>` / `RWTexture2D<float4>` become `Texture2D` /
     `RWTexture2D` (the shim's textures are RGBA float).
  6. File-scope `static const T name = expr;` resource handles become
     `#define name (expr)`: HLSL evaluates them per thread from the current
     constant buffer, a C++ static would evaluate them once at load time.
  7. Floating literals without a suffix get an `f`: an HLSL literal takes the
     precision of the float operand it meets (DXC's literal typing), while a
     C++ double literal would promote the whole expression to double.
     (Literal-only sub-expressions such as `2.0 * PI` are exact in either.)
  8. Vector / matrix constructor calls `float3(a, b, c)` become list
     initialisation `float3{a, b, c}`: C++ evaluates function arguments in an
     unspecified order, a braced list left to right as DXC does — this fixes
     the order of the two rand_float draws of
     `float2(rand_float(seed), rand_float(seed))` (wavefront/shade.hlsl:111).

Usage: python hlsl_to_cpp.py <reference_root> <out_dir>
"""
import os
import re
import sys

SHADER_DIR = os.path.join("source", "renderer", "shaders")

_FLOAT_LITERAL = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")
_INOUT = re.compile(r"\binout\s+([A-Za-z_][\w:]*(?:\s*<[^<>]*>)?)\s+([A-Za-z_]\w*)")
_ZERO_CAST = re.compile(r"\(\s*([A-Za-z_]\w*)\s*\)\s*0(?![\w.xX])")
_REGISTER = re.compile(r"\s*:\s*register\s*\([^)]*\)")
_SEMANTIC = re.compile(r"\s*:\s*SV_\w+")
_ATTRIBUTE = re.compile(r"\[\s*(?:numthreads\s*\([^)]*\)|branch|flatten|unroll|loop)\s*\]")
_TEXTURE_T = re.compile(r"\b(RW)?Texture2D\s*<\s*float4\s*>")
_STATIC_CONST = re.compile(r"^static\s+const\s+[\w<>\s]+?\s+([A-Za-z_]\w*)\s*=\s*(.*);\s*$", re.M)
_CTOR = re.compile(r"(?<![\w.])(?:float|uint|int|bool)[234](?:x[234])?\s*\(")


def _braces(text):
    out = []
    i = 0
    while True:
        m = _CTOR.search(text, i)
        if not m:
            out.append(text[i:])
            break
        open_at = m.end() - 1
        depth, j = 0, open_at
        while j < len(text):
            if text[j] == "(":
                depth += 1
            elif text[j] == ")":
                depth -= 1
                if depth == 0:
                    break
            j += 1
        if j >= len(text):
            raise ValueError("unbalanced constructor call near: " + text[m.start():m.start() + 60])
        out.append(text[i:open_at] + "{")
        # the arguments may hold further constructor calls: rewrite them too
        out.append(_braces(text[open_at + 1:j]))
        out.append("}")
        i = j + 1
    return "".join(out)


def rewrite(text):
    text = _INOUT.sub(r"\1& \2", text)
    text = _ZERO_CAST.sub(r"\1{}", text)
    text = _REGISTER.sub("", text)
    text = _SEMANTIC.sub("", text)
    text = _ATTRIBUTE.sub("", text)
    text = _TEXTURE_T.sub(lambda m: (m.group(1) or "") + "Texture2D", text)
    text = _STATIC_CONST.sub(r"#define \1 (\2)", text)
    text = _FLOAT_LITERAL.sub(lambda m: m.group(1) + "f", text)
    text = _braces(text)
    return text


def main(ref_root, out_dir):
    src = os.path.join(ref_root, SHADER_DIR)
    n = 0
    for sub in ("", "wavefront"):
        d = os.path.join(src, sub)
        for name in sorted(os.listdir(d)):
            if not (name.endswith(".hlsl") or name.endswith(".hlsl.h")):
                continue
            with open(os.path.join(d, name), encoding="utf-8") as f:
                text = f.read()
            dst_dir = os.path.join(out_dir, sub)
            os.makedirs(dst_dir, exist_ok=True)
            with open(os.path.join(dst_dir, name), "w", encoding="utf-8") as f:
                f.write(rewrite(text))
            n += 1
    print(f"rewrote {n} shader files into {out_dir}")


if __name__ == "__main__":
    if len(sys.argv) != 3:
        sys.exit(__doc__)
    main(sys.argv[1], sys.argv[2])
