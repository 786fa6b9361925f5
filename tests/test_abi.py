"""The C-ABI library builds, loads and exports every symbol include/*.h declares.
Runs without a GPU (no compute calls)."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(gbpx_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gbpx_bp_update" in syms and len(syms) >= 8


def test_library_exports_every_declared_symbol(gbpx_built):
    lib = ctypes.CDLL(gbpx_built)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_no_visible_internal_symbols(gbpx_built):
    # Only the C ABI is exported (hidden visibility for everything else).
    out = os.popen("nm -D --defined-only %s" % gbpx_built).read()
    exported = [l.split()[-1] for l in out.splitlines() if " T " in l]
    assert exported and all(s.startswith("gbpx_") for s in exported), [s for s in exported if not s.startswith("gbpx_")][:10]


def declared_arity():
    """Parameter count of every gbpx_* function declared in include/*.h."""
    arity = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for name, args in re.findall(r"\b(gbpx_\w+)\s*\(([^)]*)\)\s*;", text):
            args = args.strip()
            arity[name] = 0 if args in ("", "void") else args.count(",") + 1
    return arity


def test_python_bindings_match_header_arity(gbpx_built):
    """Every ctypes prototype the Python mirror installs has the header's parameter count."""
    from physx_gb300 import broadphase, contacts, lib, scene, server, solver, world
    for mod in (broadphase, contacts, scene, server, solver, world):
        mod._setup()
    L = lib()
    arity = declared_arity()
    checked = 0
    for name, n in arity.items():
        fn = getattr(L, name)
        if getattr(fn, "argtypes", None) is not None:
            assert len(fn.argtypes) == n, (name, len(fn.argtypes), n)
            checked += 1
    assert checked >= 20, checked


def test_immediate_library_exports_the_reference_entry_points(gbpx_built):
    """libgbpx_immediate.so exports, with C linkage, every physx::immediate entry
    point include/gbpx_immediate.h declares, and nothing else."""
    text = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "gbpx_immediate.h")).read(), flags=re.S)
    block = text[text.index('extern "C"'):]
    declared = sorted(set(re.findall(r"\b(Px\w+)\s*\(", block)))
    assert len(declared) == 22, declared
    lib = os.path.join(os.path.dirname(gbpx_built), "libgbpx_immediate.so")
    out = os.popen("nm -D --defined-only %s" % lib).read()
    exported = sorted(l.split()[-1] for l in out.splitlines() if " T " in l)
    assert exported == declared, (exported, declared)


def test_broadphase_filter_groups_and_descriptor_checks(gbpx_built):
    """PxGetBroadPhase{Static,Dynamic,Kinematic}FilterGroup give the reference's
    groups (Bp::getFilterGroup_Statics / _Dynamics, BpFiltering.h:79-89: statics 0,
    otherwise ((id + 1) << 3) | type with kinematic 1, dynamic 2), and
    PxCreateBroadPhase returns NULL for a type it does not serve (no device work)."""
    import ctypes
    lib = ctypes.CDLL(os.path.join(os.path.dirname(gbpx_built), "libgbpx_immediate.so"))
    for name in ("PxGetBroadPhaseStaticFilterGroup", "PxGetBroadPhaseDynamicFilterGroup", "PxGetBroadPhaseKinematicFilterGroup"):
        getattr(lib, name).restype = ctypes.c_uint32
    assert lib.PxGetBroadPhaseStaticFilterGroup() == 0
    for i in (0, 1, 7, 123456):
        assert lib.PxGetBroadPhaseDynamicFilterGroup(ctypes.c_uint32(i)) == ((i + 1) << 3) | 2
        assert lib.PxGetBroadPhaseKinematicFilterGroup(ctypes.c_uint32(i)) == ((i + 1) << 3) | 1

    class Desc(ctypes.Structure):   # PxBroadPhaseDesc
        _fields_ = [("mType", ctypes.c_int), ("mContextID", ctypes.c_uint64), ("mContextManager", ctypes.c_void_p),
                    ("mFoundLostPairsCapacity", ctypes.c_uint32), ("mDiscardStaticVsKinematic", ctypes.c_bool),
                    ("mDiscardKinematicVsKinematic", ctypes.c_bool)]
    lib.PxCreateBroadPhase.restype = ctypes.c_void_p
    for t in (0, 1, 4, 5):   # eSAP, eMBP, eGPU, eLAST
        assert lib.PxCreateBroadPhase(ctypes.byref(Desc(mType=t))) is None


def test_profiler_zone_callbacks(gbpx_built):
    """gbpx_set_profiler_callback: every library call opens a zone, reported to the
    user's zoneStart / zoneEnd pair (the PxProfilerCallback protocol: zoneEnd gets
    zoneStart's return value).  An invalid call still reports its zone, so no GPU
    is needed here."""
    import ctypes
    from physx_gb300 import lib
    L = lib()
    events = []
    START = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p)
    END = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p)

    def start(name, detached, ctx, user):
        events.append(("start", name.decode()))
        return 1234

    def end(data, name, detached, ctx, user):
        events.append(("end", name.decode(), data))

    s_cb, e_cb = START(start), END(end)
    L.gbpx_set_profiler_callback.argtypes = [START, END, ctypes.c_void_p]
    assert L.gbpx_set_profiler_callback(s_cb, e_cb, None) == 0
    L.gbpx_bp_update.argtypes = [ctypes.c_void_p] * 11
    assert L.gbpx_bp_update(None, None, 0, None, 0, None, 0, None, None, None, 0) == -1
    assert L.gbpx_set_profiler_callback(START(), END(), None) == 0   # removed
    assert L.gbpx_bp_update(None, None, 0, None, 0, None, 0, None, None, None, 0) == -1
    assert events == [("start", "gbpx::bp::update"), ("end", "gbpx::bp::update", 1234)]
