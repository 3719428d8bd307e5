"""Checker-build step — TEST INFRASTRUCTURE ONLY.

Writes the definitions of named host/device functions of one reference source file
(a CUDA translation unit whose kernels cannot be compiled on the host) into an include
file under oracle/_ref/, each preceded by a #line directive that points back at the
reference file, so that the checker build (oracle/ref_vbd.cpp) compiles the reference's
own function bodies unchanged. Nothing is written into the repository's sources.

Usage: python extract_ref.py SOURCE OUTPUT NAME [NAME ...]
A definition is the line that names `NAME(` (optionally `GAIA::NAME(`) outside a comment,
a preceding `template<...>` line if there is one, and everything up to the brace that
closes the function body (braces inside comments and string literals are not counted).

       python extract_ref.py --host-header HEADER OUTPUT
writes the header unchanged except that definitions written inside `namespace GAIA { }`
with a redundant `GAIA::` qualifier (accepted by MSVC, rejected by GCC) lose it.
"""
import re
import sys


def _strip_code(text: str) -> str:
    """The text with comments and string/char literals blanked (same length, same lines)."""
    out = list(text)
    i, n = 0, len(text)
    while i < n:
        c = text[i]
        if text.startswith("//", i):
            j = text.find("\n", i)
            j = n if j < 0 else j
            for k in range(i, j):
                out[k] = " "
            i = j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            j = n if j < 0 else j + 2
            for k in range(i, j):
                if text[k] != "\n":
                    out[k] = " "
            i = j
        elif c in "\"'":
            j = i + 1
            while j < n and text[j] != c:
                j += 2 if text[j] == "\\" else 1
            for k in range(i + 1, min(j, n)):
                out[k] = " "
            i = j + 1
        else:
            i += 1
    return "".join(out)


def extract(src: str, names: list[str]) -> str:
    text = open(src).read()
    code = _strip_code(text)
    lines_at = [0]
    for m in re.finditer("\n", text):
        lines_at.append(m.end())
    out = []
    for name in names:
        pat = re.compile(r"^[^\n]*?\b(?:GAIA::)?" + re.escape(name) + r"\s*\(", re.M)
        found = None
        for m in pat.finditer(code):
            start = m.start()
            # a definition: the first '{' after the parameter list comes before any ';'
            depth, j = 0, m.end() - 1
            while j < len(code):
                if code[j] == "(":
                    depth += 1
                elif code[j] == ")":
                    depth -= 1
                    if depth == 0:
                        break
                j += 1
            k = j + 1
            while k < len(code) and code[k] in " \t\r\n":
                k += 1
            if k < len(code) and code[k] == "{":
                found = (start, k)
                break
        if not found:
            raise SystemExit(f"definition of {name} not found in {src}")
        start, brace = found
        prev = text.rfind("\n", 0, max(start - 1, 0))
        prev_line = text[prev + 1:start].strip()
        if prev_line.startswith("template"):
            start = prev + 1
        depth, j = 0, brace
        while j < len(code):
            if code[j] == "{":
                depth += 1
            elif code[j] == "}":
                depth -= 1
                if depth == 0:
                    break
            j += 1
        line_no = sum(1 for a in lines_at if a <= start)
        out.append(f'#line {line_no} "{src}"\n{text[start:j + 1]}\n')
    return "".join(out)


def host_header(src: str) -> str:
    text = open(src).read()
    fixed = re.sub(r"^(\s*GPU_CPU_INLINE_FUNC\b[^\n(]*?)\bGAIA::", r"\1", text, flags=re.M)
    return f'#line 1 "{src}"\n' + fixed


if __name__ == "__main__":
    if len(sys.argv) == 4 and sys.argv[1] == "--host-header":
        with open(sys.argv[3], "w") as f:
            f.write("// generated by oracle/extract_ref.py from the reference tree; not a repository source\n")
            f.write(host_header(sys.argv[2]))
        raise SystemExit(0)
    if len(sys.argv) < 4:
        raise SystemExit(__doc__)
    body = extract(sys.argv[1], sys.argv[3:])
    with open(sys.argv[2], "w") as f:
        f.write("// generated by oracle/extract_ref.py from the reference tree; not a repository source\n")
        f.write(body)
