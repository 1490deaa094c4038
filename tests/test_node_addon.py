"""The Node-API addon and its TypeScript shim against the C ABI (CPU only).

Node and its headers are not installed here, so the addon is checked three
ways: every gs3d_* call in it names a function include/gs3d.h declares, with
that function's number of parameters; the C source compiles (-Wall -Wextra
-Werror) against declarations of the Node-API functions it uses, in Node's
signatures (tests/node_api_stub/node_api.h), the gs3d header and the CUDA
runtime header; and every native method the TypeScript shim calls is one the
addon registers.
"""
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

NODE = os.path.join(ROOT, "3dgs_tile_webgpu_gb300", "node")
ADDON = os.path.join(NODE, "gs3d_node.c")
SHIM = os.path.join(NODE, "index.ts")
HEADER = os.path.join(ROOT, "include", "gs3d.h")


def split_top_level(args: str) -> list[str]:
    out, depth, cur = [], 0, []
    for ch in args:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    tail = "".join(cur).strip()
    if tail:
        out.append(tail)
    return [a.strip() for a in out]


def header_arity() -> dict:
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    arity = {}
    for m in re.finditer(r"\b(gs3d_\w+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        params = split_top_level(m.group(2))
        arity[m.group(1)] = 0 if params in ([], ["void"]) else len(params)
    return arity


def calls(source: str):
    for m in re.finditer(r"\b(gs3d_\w+)\s*\(", source):
        i, depth = m.end(), 1
        while depth:
            depth += {"(": 1, ")": -1}.get(source[i], 0)
            i += 1
        yield m.group(1), split_top_level(source[m.end():i - 1])


def test_every_addon_call_matches_the_header():
    arity = header_arity()
    assert len(arity) >= 30
    text = re.sub(r"/\*.*?\*/", "", open(ADDON).read(), flags=re.S)
    seen = set()
    for name, args in calls(text):
        assert name in arity, f"{name} is not declared in include/gs3d.h"
        assert len(args) == arity[name], (name, args)
        seen.add(name)
    # The addon drives the whole data path of GaussianPass.
    for needed in ("gs3d_pipeline_create", "gs3d_pipeline_update_data", "gs3d_pipeline_resize_intersections",
                   "gs3d_pipeline_prepare_frame", "gs3d_pipeline_render", "gs3d_pipeline_request_stats",
                   "gs3d_pipeline_poll_stats", "gs3d_pipeline_get_resources", "gs3d_pipeline_destroy",
                   "gs3d_capacity_next"):
        assert needed in seen, needed


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_addon_compiles_against_node_api_declarations():
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not os.path.exists(os.path.join(cuda_inc, "cuda_runtime_api.h")):
        pytest.skip("CUDA runtime header not found")
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
           "-I", os.path.join(ROOT, "tests", "node_api_stub"), "-I", os.path.join(ROOT, "include"),
           "-I", cuda_inc, "-DNODE_GYP_MODULE_NAME=gs3d_node", ADDON]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def registered_methods() -> set:
    text = open(ADDON).read()
    names = set(re.findall(r'\{"(\w+)", NULL, \w+, NULL, NULL, NULL, napi_default, NULL\}', text))
    names |= set(re.findall(r'napi_set_named_property\(env, exports, "(\w+)"', text))
    return names


def test_shim_calls_only_registered_methods():
    names = registered_methods()
    assert {"render", "readStats", "prepareFrame", "createScene", "Pipeline"} <= names
    shim = open(SHIM).read()
    used = set(re.findall(r"this\.native\.(\w+)\(", shim)) | set(re.findall(r"\baddon\.(\w+)\b", shim))
    assert used, "the shim calls no native method"
    missing = used - names
    assert not missing, missing


def test_render_enqueues_only():
    # render() must not synchronise or copy (the reference's render is
    # encode-only and never blocks): the addon's render body calls no
    # blocking CUDA function.
    text = open(ADDON).read()
    body = text[text.index("static napi_value pipeline_render("):]
    body = body[:body.index("\n}\n")]
    for blocking in ("cudaStreamSynchronize", "cudaDeviceSynchronize", "cudaMemcpy(", "gs3d_pipeline_read_stats"):
        assert blocking not in body, blocking
