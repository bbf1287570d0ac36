"""Replay golden cases through any library with the builtin C ABI."""
import json

import numpy as np

from horsepower_gb300.abi import H_G, H_N, BuiltinError


def build_arg(lib, spec):
    kind = spec[0]
    if kind == "vec":
        return lib.vec(spec[1], spec[2])
    if kind == "scalar":
        return lib.scalar(spec[1], spec[2])
    if kind == "sym":
        return lib.sym(spec[1])
    if kind == "syms":
        return lib.syms(spec[1])
    if kind == "list":
        return lib.list([build_arg(lib, s) for s in spec[1]])
    if kind == "strs":
        return lib.strs(list(spec[1]))
    if kind == "chars":
        return lib.chars(spec[1])
    raise ValueError(kind)


AGGS = ["pfnSum", "pfnAvg", "pfnMin", "pfnMax", "pfnLen"]


def run_case(lib, case, fused=False):
    """Returns (rc, output object).  `fused` routes the group-aggregate chain
    through the hgpuGroup* entry points instead of each_right/each/raze."""
    args = [build_arg(lib, a) for a in case["args"]]
    fn = case["fn"]
    try:
        if fn == "@chain_group_agg":
            g = lib.call("pfnGroup", args[0])
            vals = lib.call("pfnValues", g)
            outs = []
            for agg in AGGS:
                if fused:
                    name = {"pfnSum": "hgpuGroupSum", "pfnAvg": "hgpuGroupAvg", "pfnMin": "hgpuGroupMin",
                            "pfnMax": "hgpuGroupMax", "pfnLen": "hgpuGroupLen"}[agg]
                    outs.append(lib.to_py(lib.call(name, args[1], vals)))
                else:
                    t = lib.call("pfnEachRight", args[1], vals, lib.fn_ptr("pfnIndex"))
                    e = lib.call("pfnEach", t, lib.fn_ptr(agg))
                    outs.append(lib.to_py(lib.call("pfnRaze", e)))
            return 0, outs
        if fn == "@chain_enum":
            # x: key column, y: foreign-key column, m: mask over y, pm: mask over x.
            # The foreign-key step of a plan: values, a semi-join mask through
            # the index, the kept indices and the gathered key column.
            e = lib.call("pfnEnum", args[0], args[1])
            idx = lib.call("pfnValues", e)
            kept = lib.call("pfnCompress", args[2], idx)
            from horsepower_gb300.abi import V0
            keycol = V0.from_address(args[0].g) if args[0].typ == H_G else args[0]  # first key column
            outs = [lib.to_py(idx), lib.to_py(lib.call("pfnFetch", e)), lib.to_py(lib.call("pfnKeys", e)),
                    lib.to_py(lib.call("pfnLen", e)), lib.to_py(lib.call("pfnIndex", args[3], idx)),
                    lib.to_py(kept), lib.to_py(lib.call("pfnIndex", keycol, kept))]
            return 0, outs
        z = lib.call(fn, *args)
        return 0, lib.to_py(z)
    except BuiltinError as e:
        return e.code, None


def flatten(obj):
    """Object -> (structure string, list of arrays); lists of same-dtype vectors
    are stored as one concatenation plus lengths."""
    arrays = []

    def rec(o):
        if isinstance(o, np.ndarray):
            arrays.append(o)
            return "v"
        if isinstance(o, tuple) and o and o[0] == "dict":
            return "d(" + rec(o[1]) + "," + rec(o[2]) + ")"
        if isinstance(o, list):
            if o and all(isinstance(e, np.ndarray) for e in o) and len({e.dtype for e in o}) == 1:
                arrays.append(np.concatenate(o) if o else np.zeros(0))
                arrays.append(np.array([len(e) for e in o], np.int64))
                return "c"
            return "l[" + ",".join(rec(e) for e in o) + "]"
        raise TypeError(type(o))

    return rec(obj), arrays


def store(case, rc, obj, out):
    """Serialise one case into the dict passed to np.savez_compressed."""
    name = case["name"]
    meta = dict(fn=case["fn"], tol=case["tol"], canonical=case["canonical"], error=case["error"], rc=rc)
    # inputs
    ins = []

    def enc(spec):
        if spec[0] == "vec":
            k = f"{name}/in{len(ins)}"
            ins.append(k)
            out[k] = np.asarray(spec[1])
            return ["vec", k, int(spec[2])]
        if spec[0] == "scalar":
            return ["scalar", float(spec[1]) if isinstance(spec[1], float) else int(spec[1]), int(spec[2])]
        if spec[0] == "sym":
            return ["sym", spec[1]]
        if spec[0] == "syms":
            return ["syms", list(spec[1])]
        if spec[0] == "list":
            return ["list", [enc(s) for s in spec[1]]]
        if spec[0] in ("strs", "chars"):
            k = f"{name}/in{len(ins)}"
            ins.append(k)
            texts = list(spec[1]) if spec[0] == "strs" else [spec[1]]
            out[k] = np.frombuffer(b"".join(texts), np.uint8) if texts and any(texts) else np.zeros(0, np.uint8)
            out[k + "_len"] = np.array([len(t) for t in texts], np.int64)
            return [spec[0], k]
        raise ValueError(spec)

    meta["args"] = [enc(a) for a in case["args"]]
    if obj is not None:
        struct, arrays = flatten(obj)
        meta["struct"] = struct
        meta["nout"] = len(arrays)
        for i, a in enumerate(arrays):
            out[f"{name}/out{i}"] = a
    out[f"{name}/meta"] = np.array(json.dumps(meta))


def load(path):
    """golden.npz -> list of case dicts with decoded args and expected outputs."""
    z = np.load(path, allow_pickle=False)
    names = sorted({k.split("/")[0] for k in z.files})
    cases = []
    for name in names:
        meta = json.loads(str(z[f"{name}/meta"]))

        def dec(spec):
            if spec[0] == "vec":
                return ("vec", z[spec[1]], spec[2])
            if spec[0] == "scalar":
                return ("scalar", spec[1], spec[2])
            if spec[0] == "sym":
                return ("sym", spec[1])
            if spec[0] == "syms":
                return ("syms", spec[1])
            if spec[0] in ("strs", "chars"):
                raw, lens = z[spec[1]].tobytes(), z[spec[1] + "_len"]
                texts, o = [], 0
                for n in lens:
                    texts.append(raw[o:o + int(n)])
                    o += int(n)
                return ("strs", texts) if spec[0] == "strs" else ("chars", texts[0])
            return ("list", [dec(s) for s in spec[1]])

        case = dict(name=name, fn=meta["fn"], tol=meta["tol"], canonical=meta["canonical"],
                    error=meta["error"], rc=meta["rc"], args=[dec(a) for a in meta["args"]])
        if "struct" in meta:
            case["struct"] = meta["struct"]
            case["expect"] = [z[f"{name}/out{i}"] for i in range(meta["nout"])]
        cases.append(case)
    return cases


def _canon_groups(struct, arrays):
    """Partition of a @group dict as a sorted tuple of sorted row tuples."""
    assert struct == "d(v,c)", struct
    cat, lens = arrays[1], arrays[2]
    groups, off = [], 0
    for n in lens:
        groups.append(tuple(sorted(cat[off:off + n].tolist())))
        off += n
    return sorted(groups)


def compare(case, rc, obj):
    """Raises AssertionError with a reason when `obj` does not match the fixture."""
    name = case["name"]
    if case["rc"] != 0:
        assert rc == case["rc"], f"{name}: rc {rc} != expected {case['rc']}"
        return
    assert rc == 0, f"{name}: rc {rc}"
    struct, arrays = flatten(obj)
    assert struct == case["struct"], f"{name}: structure {struct} != {case['struct']}"
    exp = case["expect"]
    if case["canonical"]:
        if struct == "d(v,c)":
            assert _canon_groups(struct, arrays) == _canon_groups(struct, exp), f"{name}: partitions differ"
            return
        # @order: the permuted values must match (tied rows may be in another order)
        x = case["args"][0][1]
        assert np.array_equal(x[arrays[0]], x[exp[0]]), f"{name}: ordered values differ"
        assert np.array_equal(np.sort(arrays[0]), np.arange(len(x))), f"{name}: not a permutation"
        return
    for i, (a, e) in enumerate(zip(arrays, exp)):
        assert a.dtype == e.dtype or a.size == 0, f"{name}: out{i} dtype {a.dtype} != {e.dtype}"
        assert a.shape == e.shape, f"{name}: out{i} shape {a.shape} != {e.shape}"
        if case["tol"] and a.dtype.kind == "f":
            ok = np.allclose(a, e, rtol=case["tol"], atol=0, equal_nan=True)
            assert ok, f"{name}: out{i} not within rtol {case['tol']}: max rel err " \
                       f"{np.max(np.abs(a - e) / np.maximum(np.abs(e), 1e-300))}"
        else:
            assert np.array_equal(a, e, equal_nan=a.dtype.kind == "f"), \
                f"{name}: out{i} differs at {np.flatnonzero(a != e)[:5]}"
