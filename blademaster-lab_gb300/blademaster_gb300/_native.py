"""Build and load the sm_103a C-ABI library (include/blademaster_gb300.h).

The ctypes structures are generated from the C header itself, so the Python
side and the compiled library cannot disagree on field order; their sizes
are checked against the library on load.  There is no CPU fallback: when
the library cannot be built or loaded, every solver call raises.
"""

import ctypes
import os
import re
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
CSRC = PACKAGE.parent / "csrc"
HEADER = PACKAGE.parent.parent / "include" / "blademaster_gb300.h"
LIBDIR = PACKAGE / "_lib"
LIBRARY = LIBDIR / "libbm_gb300.so"
SOURCES = ["bm_material.cu", "bm_contact.cu", "bm_tool.cu", "bm_hold.cu", "bm_mls.cu", "bm_mlp.cu", "bm_capi.cu", "bm_noalloc.cu", "bm_mathprobe.cu", "bm_observe.cu", "bm_embed.cu", "bm_topocut.cu"]
DEPENDS = ["bm_scalar.h", "bm_device.cuh", "bm_internal.h"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [ARCH, "-std=c++17", "-O3", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]

_lock = threading.Lock()
_lib = None


def nvcc():
    for candidate in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if candidate and (Path(candidate).exists() or candidate == "nvcc"):
            return candidate
    raise RuntimeError("nvcc not found")


def _stale():
    if not LIBRARY.exists():
        return True
    built = LIBRARY.stat().st_mtime
    inputs = [CSRC / f for f in SOURCES + DEPENDS] + [HEADER]
    return any(p.stat().st_mtime > built for p in inputs)


def build(force=False, verbose=False):
    """Compile every .cu for sm_103a (in parallel) and link the shared library."""
    with _lock:
        if not force and not _stale():
            return LIBRARY
        LIBDIR.mkdir(exist_ok=True)
        objects = [LIBDIR / (Path(s).stem + ".o") for s in SOURCES]
        logs = {}

        def compile_one(args):
            src, obj = args
            cmd = [nvcc(), *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            logs[src] = r.stdout + r.stderr
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")

        with ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
            list(pool.map(compile_one, zip(SOURCES, objects)))
        tmp = LIBRARY.with_suffix(".so.tmp")
        cmd = [nvcc(), ARCH, "-shared", "-o", str(tmp), *map(str, objects)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIBRARY)
        (LIBDIR / "ptxas.log").write_text("\n".join(f"== {k}\n{v}" for k, v in logs.items()))
        if verbose:
            print((LIBDIR / "ptxas.log").read_text())
        return LIBRARY


# ------------------------------------------------------- header-driven structs

_CTYPES = {
    "int32_t": ctypes.c_int32,
    "int64_t": ctypes.c_int64,
    "uint64_t": ctypes.c_uint64,
    "float": ctypes.c_float,
    "double": ctypes.c_double,
}


def _struct_fields(name):
    text = HEADER.read_text()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = re.sub(r"^const\s+", "", decl.strip())
        if not decl:
            continue
        m = re.match(r"(\w+)\s*(\*?)\s*(.*)", decl)
        ctype, pointer, names = m.group(1), m.group(2), m.group(3)
        for item in names.split(","):
            item = item.strip()
            if item.startswith("*"):
                pointer, item = "*", item[1:].strip()
            arr = re.match(r"(\w+)\[(\d+)\]", item)
            if pointer:
                fields.append((item, ctypes.c_void_p))
            elif arr:
                fields.append((arr.group(1), _CTYPES[ctype] * int(arr.group(2))))
            else:
                fields.append((item, _CTYPES[ctype]))
    return fields


class Params(ctypes.Structure):
    _fields_ = _struct_fields("bm_params")


class Buffers(ctypes.Structure):
    _fields_ = _struct_fields("bm_buffers")


class StepArgs(ctypes.Structure):
    _fields_ = _struct_fields("bm_step_args")


class MlsParams(ctypes.Structure):
    _fields_ = _struct_fields("bm_mls_params")


class MlsBuffers(ctypes.Structure):
    _fields_ = _struct_fields("bm_mls_buffers")


class Embedding(ctypes.Structure):
    _fields_ = _struct_fields("bm_embedding")


class TopoCutGrid(ctypes.Structure):
    _fields_ = _struct_fields("bm_topocut_grid")


def header_constant(name):
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    m = re.search(r"#define %s \(?([^\n]+)" % name, text)
    return m.group(1).strip().rstrip(")")


PAIR_LANES = int(header_constant("BM_PAIR_LANES"))
MAX_TOOLS = int(header_constant("BM_MAX_TOOLS"))
TOOL_F_WORDS = int(header_constant("BM_TOOL_F_WORDS"))
FLAG = {
    k: int(header_constant("BM_FLAG_" + k))
    for k in ("TOPOLOGY_DIRTY", "PAIR_DIRTY", "PAIR_BUILDS", "STEP", "CANDIDATES", "EMBEDDED", "SLOTS", "CHANGED",
              "RELIST", "MULTI", "RELISTS", "MIXED_CELLS", "REGISTRATIONS", "MAX_DISP", "HOLD_NEEDS",
              "HOLD_RESIDUAL", "HOLD_COUNT", "HOLD_NODES", "REG_MODE", "REG_CHANGED", "REG_NODES", "REG_CELLS",
              "HOST_DIRTY", "PAIR_SPEED", "WORDS")
}
CUT_ON, CUT_ADVANCE, CUT_HOLD = 1, 2, 4
STAGES = ["prologue", "rigid", "pairs", "register", "p2g", "g2p", "remap", "tool", "fupdate", "assign"]
ACC_WORDS = 2 * (6 * MAX_TOOLS + 4)


def _declare(lib):
    vp, i, f, u64p = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_void_p
    sigs = {
        "bm_params_size": ([], ctypes.c_uint32),
        "bm_buffers_size": ([], ctypes.c_uint32),
        "bm_step_args_size": ([], ctypes.c_uint32),
        "bm_last_error": ([], ctypes.c_char_p),
        "bm_version": ([], ctypes.c_char_p),
        "bm_scratch_words": ([ctypes.POINTER(Params)], ctypes.c_int64),
        "bm_solver_create": ([ctypes.POINTER(Params), ctypes.POINTER(Buffers), ctypes.POINTER(vp)], i),
        "bm_solver_destroy": ([vp], i),
        "bm_refresh_stress": ([vp, vp], i),
        "bm_register_topology": ([vp, i, vp], i),
        "bm_material_step": ([vp, i, vp], i),
        "bm_rigid_contacts": ([vp, i, vp], i),
        "bm_particle_contacts": ([vp, vp], i),
        "bm_particle_contacts_static": ([vp, vp], i),
        "bm_hold_constraint": ([vp, vp], i),
        "bm_gemm_tn_bf16": ([vp, vp, vp, i, i, i, vp, i, vp, vp, vp], i),
        "bm_gemm_set_loop_wait_limit": ([ctypes.c_longlong], i),
        "bm_mlp_transpose16": ([vp, vp, i, i, vp], i),
        "bm_mlp_relu_grad": ([vp, vp, vp, ctypes.c_int64, vp], i),
        "bm_mlp_pool": ([vp, i, vp, f, f, vp, vp], i),
        "bm_mlp_mse_grad": ([vp, vp, i, i, i, vp, vp, vp, vp], i),
        "bm_mlp_colsum": ([vp, i, i, vp, vp], i),
        "bm_mlp_cast_bf16": ([vp, i, i, i, vp, vp], i),
        "bm_mlp_adam": ([vp, vp, vp, vp, vp, ctypes.c_int64, f, f, f, f, i, vp], i),
        "bm_mls_create": ([ctypes.POINTER(MlsParams), ctypes.POINTER(MlsBuffers), ctypes.POINTER(Params),
                           ctypes.POINTER(Buffers), ctypes.POINTER(vp)], i),
        "bm_mls_destroy": ([vp], i),
        "bm_mls_substeps": ([vp, i, vp], i),
        "bm_mls_graph_create": ([vp, i, vp, ctypes.POINTER(vp)], i),
        "bm_assign_sides": ([vp, i, i, vp], i),
        "bm_drive_tool": ([vp, i, vp], i),
        "bm_finish_external": ([vp, vp], i),
        "bm_accumulate_tool_impulses": ([vp, vp], i),
        "bm_clear_step": ([vp, vp], i),
        "bm_substeps": ([vp, ctypes.POINTER(StepArgs), vp], i),
        "bm_graph_create": ([vp, ctypes.POINTER(StepArgs), vp, ctypes.POINTER(vp)], i),
        "bm_substeps_profiled": ([vp, ctypes.POINTER(StepArgs), vp, vp], i),
        "bm_graph_launch": ([vp, vp], i),
        "bm_batch_graph_create": ([ctypes.POINTER(vp), ctypes.POINTER(StepArgs), i, i, vp, ctypes.POINTER(vp)], i),
        "bm_graph_destroy": ([vp], i),
        "bm_graph_kernel_count": ([vp, ctypes.POINTER(ctypes.c_int64)], i),
        "bm_metrics": ([vp, vp, vp], i),
        "bm_components": ([vp, vp, vp, vp, vp, vp, vp], i),
        "bm_embed_nodes": ([vp, vp, vp, vp, vp, ctypes.c_int64, i, vp, vp, vp, vp], i),
        "bm_embed_vertices": ([vp, i, vp, vp, vp, vp, vp, vp, vp, vp, vp], i),
        "bm_topocut_sdf": ([vp, vp, i, vp, vp, vp, vp, vp, vp, vp], i),
        "bm_topocut_count": ([vp, vp, vp, vp, vp, vp, vp, vp, vp, vp], i),
        "bm_topocut_emit": ([vp, vp, vp, vp, vp, vp, vp, vp], i),
        "bm_topocut_cluster": ([vp, i, vp, vp, vp, i, ctypes.c_float, ctypes.c_float, vp, vp], i),
        "bm_count_embedded": ([vp, i, vp], i),
        "bm_validate_interval": ([vp, vp], i),
        "bm_read_accumulators": ([vp, vp, vp, vp, vp, vp], i),
        "bm_write_accumulators": ([vp, vp, vp, vp, vp, vp], i),
        "bm_sync_tool_mirror": ([vp, vp], i),
        "bm_blade_query": ([vp, i, vp, f, vp, vp, vp, vp], i),
        "bm_friction": ([vp, vp, vp, vp, i, f, f, f, f, f, f, vp, vp, vp], i),
        "bm_couple_fields": ([vp, vp, vp, vp, i, vp, vp], i),
        "bm_g2p_probe": ([vp, vp, vp, vp, vp, vp, i, f, f, vp], i),
        "bm_resist_cut_probe": ([vp, vp, vp, vp, vp, vp, vp, vp, f, f, vp, f, i, u64p, vp, i, vp], i),
        "bm_plastic_project": ([vp, vp, i, f, f, vp, vp], i),
        "bm_math_probe_f": ([i, vp, i, vp, vp], i),
        "bm_math_probe_d": ([i, vp, vp, i, vp, vp], i),
        "bm_svd_probe": ([vp, i, vp, vp, vp, vp, vp], i),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


def exported_symbols():
    """Names of the functions the header declares (used by the ABI test)."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(bm_\w+)\s*\(", text, re.M)))


def lib():
    """The loaded library (built on first use if missing or stale)."""
    global _lib
    if _lib is None:
        build()
        loaded = _declare(ctypes.CDLL(str(LIBRARY)))
        for name, cls in (("bm_params_size", Params), ("bm_buffers_size", Buffers), ("bm_step_args_size", StepArgs)):
            if getattr(loaded, name)() != ctypes.sizeof(cls):
                raise RuntimeError(f"{name}: library and header disagree; rebuild")
        _lib = loaded
    return _lib


def check(rc):
    """Raise with the library's message on a failed call."""
    if rc != 0:
        raise RuntimeError(f"blademaster_gb300 error {rc}: {lib().bm_last_error().decode()}")
