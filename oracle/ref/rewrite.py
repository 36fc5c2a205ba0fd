"""OpenCL C -> C++20 source rewrite for the shim in clshim.h (TEST INFRASTRUCTURE ONLY).

The reference's kernel files are compiled as they are, except for the few constructs whose
C++ reading differs from OpenCL C's. This module makes exactly these textual changes and
nothing else (line numbers are preserved, so compiler messages point at the reference's
own lines through a #line directive):

1. comments are blanked (kept as spaces and newlines), so commented-out kernels are ignored;
2. vector literals `(float4)(a, b, c, d)` (and float2/int2/int4/uint2/uint4) become
   `clc::make<clc::float4>(a, b, c, d)`: in C++ the original parses as a cast of a comma
   expression and silently keeps only the last operand;
3. `__local` in a parameter list is dropped (the runner passes one buffer per work-group);
   an array `__local T name[N];` inside a kernel body becomes a reference bound once per
   work-item, `T (&name)[N] = clc::local_array<T, N, SITE>();`, to storage that the host
   thread running the work-group owns (so it is shared by the work-group, as OpenCL's local
   memory is, and later accesses need no thread-local lookup); any other `__local` inside a
   body becomes `static thread_local`;
4. a kernel whose body calls barrier() becomes a coroutine: its return type `void` becomes
   `clc::wi_task`, `barrier(...);` becomes `co_await clc::barrier_point{};` and `return;`
   becomes `co_return;`;
5. in such a kernel, a statement at the top level of the body of the form
   `a[lid] = min(a[lid], a[lid ^ k]);` (or max) -- a butterfly step that reads another
   work-item's __local element with no barrier in between, relying on the work-group being
   one 32-wide warp executing each statement in lockstep (clAABB in
   libCL/geom/oclBvhTrimesh.cl:53-60, launched with a local size of 32, cWarpSize in
   libCL/geom/oclBvhTrimesh.cpp:18,87) -- gets a barrier appended on its line, so that the
   host runs the statement for every work-item before the next one, as the warp does.
"""
from __future__ import annotations

import re

_VEC_LITERAL = re.compile(r"\(\s*(float|int|uint)(2|4)\s*\)\s*\(")
_BARRIER = re.compile(r"\bbarrier\s*\([^;]*\)\s*;")
_RETURN = re.compile(r"\breturn\s*;")
_KERNEL = re.compile(r"__kernel\s+void\s+\w+\s*\(")
_BUTTERFLY = re.compile(r"^\s*(\w+)\[(\w+)\]\s*=\s*(min|max)\(\s*\1\[\2\]\s*,\s*\1\[\2\s*\^\s*\d+\]\s*\)\s*;\s*$")


def blank_comments(src: str) -> str:
    """Replaces // and /* */ comments by spaces, keeping every newline."""
    out = []
    i, n = 0, len(src)
    while i < n:
        if src.startswith("//", i):
            j = src.find("\n", i)
            j = n if j < 0 else j
            out.append(" " * (j - i))
            i = j
        elif src.startswith("/*", i):
            j = src.find("*/", i + 2)
            j = n if j < 0 else j + 2
            out.append("".join(c if c == "\n" else " " for c in src[i:j]))
            i = j
        elif src[i] == '"':
            j = i + 1
            while j < n and src[j] != '"':
                j += 2 if src[j] == "\\" else 1
            out.append(src[i:j + 1])
            i = j + 1
        else:
            out.append(src[i])
            i += 1
    return "".join(out)


def _match(src: str, i: int, open_c: str, close_c: str) -> int:
    """Index one past the bracket that closes the one at src[i]."""
    depth = 0
    for j in range(i, len(src)):
        if src[j] == open_c:
            depth += 1
        elif src[j] == close_c:
            depth -= 1
            if depth == 0:
                return j + 1
    raise ValueError(f"unbalanced {open_c}{close_c} from offset {i}")


_LOCAL_ARRAY = re.compile(r"__local\s+(\w+)\s+(\w+)\s*\[([^\]]+)\]\s*;")


def _locals(src: str) -> str:
    out = []
    depth = 0
    site = 0
    i = 0
    for m in re.finditer(r"[{}]|\b__local\b", src):
        if m.start() < i:
            continue
        out.append(src[i:m.start()])
        tok = m.group(0)
        i = m.end()
        if tok == "{":
            depth += 1
            out.append(tok)
        elif tok == "}":
            depth -= 1
            out.append(tok)
        elif depth == 0:
            out.append("")
        else:
            arr = _LOCAL_ARRAY.match(src, m.start())
            if arr:
                t, name, n = arr.groups()
                site += 1
                out.append(f"{t} (&{name})[{n}] = clc::local_array<{t}, ({n}), {site}>();")
                i = arr.end()
            else:
                out.append("static thread_local")
    out.append(src[i:])
    return "".join(out)


def _lockstep(body: str) -> str:
    """Rule 5: a barrier after each butterfly statement at the body's top level (brace depth
    1 of the body, which starts at its opening brace)."""
    out = []
    depth = 0
    for line in body.split("\n"):
        if depth == 1 and _BUTTERFLY.match(line):
            line = line + " barrier(CLK_LOCAL_MEM_FENCE);"
        depth += line.count("{") - line.count("}")
        out.append(line)
    return "\n".join(out)


def _coroutines(src: str) -> tuple[str, list[str]]:
    out = []
    names = []
    i = 0
    for m in _KERNEL.finditer(src):
        if m.start() < i:
            continue
        p_end = _match(src, m.end() - 1, "(", ")")
        b_start = src.index("{", p_end)
        b_end = _match(src, b_start, "{", "}")
        body = src[b_start:b_end]
        out.append(src[i:m.start()])
        header = src[m.start():b_start]
        if _BARRIER.search(body):
            name = re.match(r"__kernel\s+void\s+(\w+)", header).group(1)
            names.append(name)
            body = _lockstep(body)
            header = re.sub(r"__kernel\s+void", "clc::wi_task", header, count=1)
            body = _BARRIER.sub("co_await clc::barrier_point{};", body)
            body = _RETURN.sub("co_return;", body)
        out.append(header)
        out.append(body)
        i = b_end
    out.append(src[i:])
    return "".join(out), names


def rewrite(src: str, origin: str) -> str:
    """The C++ translation unit fragment for one .cl file (to be #included inside a
    namespace nested in clc). `origin` is the reference path used in the #line directive."""
    text = blank_comments(src)
    text = _VEC_LITERAL.sub(lambda m: f"clc::make<clc::{m.group(1)}{m.group(2)}>(", text)
    text = _locals(text)
    text, coro = _coroutines(text)
    head = (f"// Generated from {origin} by oracle/ref/rewrite.py; not part of the repository.\n"
            f"// Kernels compiled as coroutines (they call barrier()): {', '.join(coro) or 'none'}\n"
            f"#line 1 \"{origin}\"\n")
    return head + text
