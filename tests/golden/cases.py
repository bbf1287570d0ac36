"""Golden-vector cases for the HorseIR builtins on the accelerated path.

Each case is a builtin name plus its arguments, built from seeded numpy
inputs.  `make_golden.py` runs every case through the reference's own
builtin library (compiled from its sources) and stores inputs and outputs in
`golden.npz`; the tests replay the stored inputs through the oracle port
(CPU suite) and through libhgpu (GPU suite) and compare.

Argument encoding (so a fixture can be rebuilt without this module):
  ("vec", array, typ) | ("scalar", value, typ) | ("sym", name) | ("syms", [names]) | ("list", [args]) | ("bools", array)
Case flags:
  tol        relative tolerance for float outputs (0 = bit-exact)
  canonical  compare a @group / @order result up to the order of tied rows
             (reference paths built on its unstable quicksort)
  error      the case is expected to return this E_* code
"""
import numpy as np

H_B, H_J, H_H, H_I, H_L, H_F, H_E, H_C, H_D = 0, 1, 2, 3, 4, 5, 6, 8, 12


def V(a, typ):
    return ("vec", np.asarray(a), typ)


def S(v, typ):
    return ("scalar", v, typ)


def Ls(*items):
    return ("list", list(items))


def build_cases():
    rng = np.random.default_rng(20261203)
    cases = []

    def add(name, fn, *args, tol=0.0, canonical=False, error=0):
        cases.append(dict(name=name, fn=fn, args=list(args), tol=tol, canonical=canonical, error=error))

    # ---- reference documentation examples (docs/mkdocs/docs/horseir/builtin/*.md)
    add("doc_compress", "pfnCompress", V([1, 1, 0], H_B), V([53, 11, 12], H_I))
    add("doc_group", "pfnGroup", V([-1, 3, 2, 3], H_I))
    add("doc_order", "pfnOrderBy", V([32, 12, 7, 78, 23, 45], H_I), V([1], H_B))

    # ---- @compress / @where (h_primitive.cc:1479-1521, :728-762)
    n = 20000
    for dens, tag in [(0.3, "r30"), (0.018, "sparse"), (0.0, "none"), (1.0, "all")]:
        m = rng.random(n) < dens
        for typ, dt in [(H_B, np.bool_), (H_J, np.int8), (H_H, np.int16), (H_I, np.int32),
                        (H_L, np.int64), (H_F, np.float32), (H_E, np.float64), (H_C, np.int8)]:
            vals = (rng.integers(-100, 100, n) if dt not in (np.float32, np.float64)
                    else rng.standard_normal(n)).astype(dt)
            add(f"compress_{tag}_{typ}", "pfnCompress", V(m, H_B), V(vals, typ))
        add(f"where_{tag}", "pfnWhere", V(m, H_B))
    add("compress_empty", "pfnCompress", V(np.zeros(0, bool), H_B), V(np.zeros(0, np.float64), H_E))
    add("compress_one", "pfnCompress", V([True], H_B), V([2.5], H_E))
    add("compress_len_mismatch", "pfnCompress", V([True, False], H_B), V([1, 2, 3], H_I), error=5)
    add("compress_not_bool", "pfnCompress", V([1, 0], H_I), V([1, 2], H_I), error=1)
    add("where_small", "pfnWhere", V(rng.random(500) < 0.5, H_B))
    add("where_odd", "pfnWhere", V(rng.random(12345) < 0.5, H_B))

    # ---- compares (h_primitive.cc:1073-1200, eps 1e-13)
    xi = rng.integers(-60, 60, n).astype(np.int32)
    xe = np.round(rng.standard_normal(n), 2)
    xe[:50] = 0.05 + np.array([0, 1e-14, -1e-14, 5e-14, -5e-14, 2e-13, -2e-13, 1e-12, -1e-12, 0] * 5)
    xe[50] = np.nan
    for op in ["pfnLt", "pfnLeq", "pfnGt", "pfnGeq", "pfnEq", "pfnNeq"]:
        add(f"{op}_i32_s", op, V(xi, H_I), S(24, H_I))
        add(f"{op}_f64_s", op, V(xe, H_E), S(0.05, H_E))
        add(f"{op}_s_f64", op, S(0.05, H_E), V(xe, H_E))
        add(f"{op}_i32_f64", op, V(xi, H_I), V(xe * 30, H_E))
        add(f"{op}_j_h", op, V(rng.integers(-5, 5, 300).astype(np.int8), H_J),
            V(rng.integers(-5, 5, 300).astype(np.int16), H_H))
        add(f"{op}_date_s", op, V(rng.integers(8000, 10526, 3000).astype(np.int32), H_D), S(8766, H_D))
        add(f"{op}_char", op, V(rng.integers(0, 120, 300).astype(np.int8), H_C),
            V(rng.integers(0, 120, 300).astype(np.int8), H_C))
        add(f"{op}_f32_s", op, V(rng.standard_normal(500).astype(np.float32), H_F), S(0.25, H_F))
    add("cmp_len_mismatch", "pfnLt", V([1, 2, 3], H_I), V([1, 2], H_I), error=5)
    add("cmp_type", "pfnLt", V([1, 2], H_I), V([1, 2], H_D), error=6)

    # ---- arithmetic (h_primitive.cc:1227-1309)
    a32 = rng.integers(-2 ** 31, 2 ** 31 - 1, 3000, dtype=np.int64).astype(np.int32)
    b32 = rng.integers(-2 ** 31, 2 ** 31 - 1, 3000, dtype=np.int64).astype(np.int32)
    b32[b32 == 0] = 7
    for op in ["pfnPlus", "pfnMinus", "pfnMul", "pfnDiv"]:
        add(f"{op}_i32", op, V(a32, H_I), V(b32, H_I))
        add(f"{op}_f64", op, V(rng.standard_normal(3000), H_E), V(rng.standard_normal(3000) + 3, H_E))
        add(f"{op}_i32_f64_s", op, V(a32, H_I), S(1.5, H_E))
        add(f"{op}_s_i64", op, S(7, H_L), V(b32.astype(np.int64), H_L))
        add(f"{op}_j", op, V(rng.integers(-128, 127, 500).astype(np.int8), H_J),
            V(rng.integers(1, 127, 500).astype(np.int8), H_J))
        add(f"{op}_b", op, V(rng.random(200) < 0.5, H_B), V(np.ones(200, bool), H_B))
        add(f"{op}_f32", op, V(rng.standard_normal(500).astype(np.float32), H_F),
            V((rng.standard_normal(500) + 4).astype(np.float32), H_F))
    add("div_zero", "pfnDiv", V([1, 2, 3], H_I), V([1, 0, 3], H_I), error=4)
    add("div_zero_f", "pfnDiv", V([1.0, 2.0], H_E), V([1.0, 0.0], H_E), error=4)
    add("mul_q6", "pfnMul", V(np.round(rng.uniform(900, 105000, 4000) * 3 / 100, 2), H_E),
        V(rng.integers(0, 11, 4000) / 100.0, H_E))

    # ---- logic (h_primitive.cc:1315-1357)
    ba, bb = rng.random(5000) < 0.5, rng.random(5000) < 0.5
    for op in ["pfnAnd", "pfnNand", "pfnOr", "pfnNor", "pfnXor"]:
        add(f"{op}_vv", op, V(ba, H_B), V(bb, H_B))
        add(f"{op}_vs", op, V(ba, H_B), S(True, H_B))
    add("not", "pfnNot", V(ba, H_B))

    # ---- reductions (h_primitive.cc:764-847)
    for typ, arr in [(H_B, rng.random(9000) < 0.5), (H_J, rng.integers(-128, 127, 9000).astype(np.int8)),
                     (H_H, rng.integers(-30000, 30000, 9000).astype(np.int16)),
                     (H_I, rng.integers(-2 ** 31, 2 ** 31 - 1, 9000, dtype=np.int64).astype(np.int32)),
                     (H_L, rng.integers(-2 ** 62, 2 ** 62, 9000, dtype=np.int64)),
                     (H_E, rng.uniform(0, 1e5, 9000)), (H_F, rng.uniform(0, 10, 9000).astype(np.float32))]:
        tol = 1e-12 if typ == H_E else (1e-5 if typ == H_F else 0.0)
        add(f"sum_{typ}", "pfnSum", V(arr, typ), tol=tol)
        add(f"avg_{typ}", "pfnAvg", V(arr, typ), tol=tol if tol else 1e-15)
        if typ != H_F:
            add(f"min_{typ}", "pfnMin", V(arr, typ))
            add(f"max_{typ}", "pfnMax", V(arr, typ))
    for typ, dt in [(H_I, np.int32), (H_E, np.float64), (H_F, np.float32)]:
        add(f"min_empty_{typ}", "pfnMin", V(np.zeros(0, dt), typ))
        add(f"max_empty_{typ}", "pfnMax", V(np.zeros(0, dt), typ))
        add(f"sum_empty_{typ}", "pfnSum", V(np.zeros(0, dt), typ))
    add("sum_one", "pfnSum", V([3.25], H_E))
    add("len", "pfnLen", V(xe, H_E))
    # min/max fold restarting after NaNs, signed zeros, infinities; sums over
    # specials and wide exponent ranges (own generator: the cases above keep
    # their inputs)
    r2 = np.random.default_rng(5150)
    for typ, dt in [(H_E, np.float64), (H_F, np.float32)]:
        pool = np.array([0.0, -0.0, 1.5, -1.5, np.inf, -np.inf, 3.0, -7.25], dt)
        mixed = pool[r2.integers(0, pool.size, 9000)]
        mixed[[17, 4100, 5000, 8190]] = np.nan
        last = mixed.copy()
        last[-1] = np.nan
        for nm, arr in [("nan_mid", mixed), ("nan_last", last), ("zeros", np.array([0.0, -0.0, 0.0, -0.0], dt)),
                        ("zeros_rev", np.array([-0.0, 0.0, -0.0], dt)), ("nan_first", np.array([np.nan, 2.0, -3.0], dt)),
                        ("one_nan", np.array([np.nan], dt))]:
            add(f"min_{nm}_{typ}", "pfnMin", V(arr, typ))
            add(f"max_{nm}_{typ}", "pfnMax", V(arr, typ))
    wide = r2.standard_normal(9000) * np.ldexp(1.0, r2.integers(-80, 80, 9000))
    add("sum_wide_exponents", "pfnSum", V(wide, H_E), tol=1e-12)
    add("avg_wide_exponents", "pfnAvg", V(wide, H_E), tol=1e-12)
    add("sum_subnormals", "pfnSum", V(np.array([5e-324, 1e-310, -2e-320, 3e-315]), H_E), tol=1e-12)
    add("sum_inf", "pfnSum", V(np.array([1.0, np.inf, 2.0]), H_E))
    add("sum_inf_minus_inf", "pfnSum", V(np.array([np.inf, 1.0, -np.inf]), H_E))
    add("sum_nan", "pfnSum", V(np.array([1.0, np.nan, 2.0]), H_E))
    add("sum_neg_zeros", "pfnSum", V(np.array([-0.0, -0.0]), H_E))

    # ---- gather (h_primitive.cc:43-94)
    src = {H_E: rng.standard_normal(7000), H_I: rng.integers(-99, 99, 7000).astype(np.int32),
           H_C: rng.integers(0, 120, 7000).astype(np.int8), H_B: rng.random(7000) < 0.5,
           H_L: rng.integers(-2 ** 40, 2 ** 40, 7000, dtype=np.int64)}
    idx = rng.integers(0, 7000, 9000).astype(np.int64)
    for typ, arr in src.items():
        add(f"index_{typ}", "pfnIndex", V(arr, typ), V(idx, H_L))
    add("index_oob", "pfnIndex", V(src[H_E], H_E), V([1, 7000], H_L), error=3)
    add("index_scalar", "pfnIndex", V(src[H_I], H_I), S(5, H_L))

    # ---- index_of (h_primitive.cc:1523-1579)
    x = rng.permutation(30000)[:8000].astype(np.int32)
    add("index_of_i32", "pfnIndexOf", V(x, H_I), V(rng.integers(0, 30000, 12000).astype(np.int32), H_I))
    dup = rng.integers(0, 500, 4000).astype(np.int64)
    add("index_of_i64_dup", "pfnIndexOf", V(dup, H_L), V(rng.integers(0, 700, 5000).astype(np.int64), H_L))
    asc = np.sort(rng.integers(0, 5000, 3000)).astype(np.int32)
    add("index_of_sorted", "pfnIndexOf", V(asc, H_I), V(rng.integers(-10, 5010, 4000).astype(np.int32), H_I))
    add("index_of_desc", "pfnIndexOf", V(asc[::-1].copy(), H_I), V(rng.integers(0, 5000, 4000).astype(np.int32), H_I))
    add("index_of_const", "pfnIndexOf", V(np.full(50, 7, np.int64), H_L), V([7, 8, 7], H_L))
    fx = np.round(rng.standard_normal(3000), 3)
    add("index_of_f64", "pfnIndexOf", V(fx, H_E), V(np.round(rng.standard_normal(3000), 3), H_E))
    add("index_of_bool", "pfnIndexOf", V(rng.random(100) < 0.7, H_B), V(rng.random(50) < 0.5, H_B))
    add("index_of_mixed", "pfnIndexOf", V(rng.integers(0, 100, 300).astype(np.int16), H_H),
        V(rng.integers(0, 120, 400).astype(np.int32), H_I))

    # ---- member (h_primitive.cc:2287-2336): pfnMember(z, probe, set)
    add("member_i32", "pfnMember", V(rng.integers(0, 3000, 9000).astype(np.int32), H_I),
        V(rng.integers(0, 3000, 1500).astype(np.int32), H_I))
    add("member_i64_small2", "pfnMember", V(rng.integers(0, 5, 400).astype(np.int64), H_L), V([1, 3], H_L))
    add("member_i64_small1", "pfnMember", V(rng.integers(0, 5, 400).astype(np.int64), H_L), V([4], H_L))
    add("member_f64", "pfnMember", V(np.round(rng.standard_normal(3000), 2), H_E),
        V(np.round(rng.standard_normal(800), 2), H_E))
    add("member_bool", "pfnMember", V(rng.random(100) < 0.5, H_B), V([True, True], H_B))
    add("member_mixed", "pfnMember", V(rng.integers(0, 100, 300).astype(np.int32), H_I),
        V(rng.integers(0, 100, 40).astype(np.int64), H_L))

    # ---- join_index (h_primitive.cc:2122-2155; hash v3 for i32 keys)
    pk = rng.permutation(40000).astype(np.int32)[:9000]
    fk = rng.integers(0, 40000, 30000).astype(np.int32)
    add("join_pk_fk", "pfnJoinIndex", V(pk, H_I), V(fk, H_I), ("sym", "eq"))
    add("join_fk_pk_swapped", "pfnJoinIndex", V(fk, H_I), V(pk, H_I), ("sym", "eq"))
    bdup = rng.integers(0, 300, 2000).astype(np.int32)
    add("join_dup_build", "pfnJoinIndex", V(bdup, H_I), V(rng.integers(0, 400, 5000).astype(np.int32), H_I), ("sym", "eq"))
    add("join_equal_len", "pfnJoinIndex", V(rng.integers(0, 50, 1000).astype(np.int32), H_I),
        V(rng.integers(0, 50, 1000).astype(np.int32), H_I), ("sym", "eq"))
    add("join_linear_small", "pfnJoinIndex", V([5, 3, 5, 9], H_I), V(rng.integers(0, 10, 500).astype(np.int32), H_I), ("sym", "eq"))
    add("join_linear_neq", "pfnJoinIndex", V([5, 3], H_I), V(rng.integers(0, 10, 50).astype(np.int32), H_I), ("sym", "neq"))
    add("join_linear_f64", "pfnJoinIndex", V([0.5, 0.25, 0.5], H_E), V(rng.integers(0, 4, 60) / 4.0, H_E), ("sym", "eq"))
    add("join_no_match", "pfnJoinIndex", V(np.arange(100, 200, dtype=np.int32), H_I), V(np.arange(0, 50, dtype=np.int32), H_I), ("sym", "eq"))
    add("join_mixed_types", "pfnJoinIndex", V(rng.permutation(500).astype(np.int16)[:200], H_H),
        V(rng.integers(0, 500, 900).astype(np.int32), H_I), ("sym", "eq"))

    # ---- group (h_primitive.cc:993-1057, 2656-2681)
    add("group_i32", "pfnGroup", V(rng.integers(0, 700, 10000).astype(np.int32), H_I))
    add("group_i32_neg", "pfnGroup", V(rng.integers(-300, 300, 6000).astype(np.int32), H_I))
    add("group_i64_small", "pfnGroup", V(rng.integers(-1000, 1000, 6000).astype(np.int64), H_L))
    add("group_i64_wide", "pfnGroup", V(rng.integers(0, 5, 4000).astype(np.int64) * (2 ** 33) + rng.integers(0, 3, 4000), H_L))
    add("group_i64_mixed_hi", "pfnGroup", V(np.array([-1, 4294967295, 5, -1, 4294967295, 7, 2 ** 40, -1], np.int64), H_L))
    add("group_sorted", "pfnGroup", V(np.sort(rng.integers(0, 90, 3000)).astype(np.int32), H_I))
    add("group_trie", "pfnGroup", Ls(V(rng.integers(0, 3, 12000).astype(np.int8), H_C), V(rng.integers(0, 2, 12000).astype(np.int8), H_C)))
    add("group_list_ii", "pfnGroup", Ls(V(rng.integers(0, 20, 5000).astype(np.int32), H_I), V(rng.integers(0, 20, 5000).astype(np.int32), H_I)))
    add("group_list_li", "pfnGroup", Ls(V(rng.integers(-30, 30, 5000).astype(np.int64), H_L), V(rng.integers(-5, 5, 5000).astype(np.int32), H_I)))
    add("group_list_jj", "pfnGroup", Ls(V(rng.integers(0, 3, 5000).astype(np.int8), H_J), V(rng.integers(0, 2, 5000).astype(np.int8), H_J)))
    add("group_f64", "pfnGroup", V(np.round(rng.standard_normal(3000), 1), H_E))
    add("group_char", "pfnGroup", V(rng.integers(0, 60, 3000).astype(np.int8), H_C))
    add("group_empty", "pfnGroup", V(np.zeros(0, np.int32), H_I))

    # ---- order (h_primitive.cc:1769-1816)
    oi = rng.integers(-50, 50, 6000).astype(np.int32)
    add("order_i32_asc", "pfnOrderBy", V(oi, H_I), V([1], H_B))
    add("order_i32_desc", "pfnOrderBy", V(oi, H_I), V([0], H_B))
    ol = rng.integers(0, 3000, 6000).astype(np.int64)
    add("order_i64_asc", "pfnOrderBy", V(ol, H_L), V([1], H_B))
    add("order_i64_desc", "pfnOrderBy", V(ol, H_L), V([0], H_B))
    add("order_case1", "pfnOrderBy", Ls(V(rng.integers(0, 40, 5000).astype(np.int32), H_I), V(rng.integers(-20, 20, 5000).astype(np.int32), H_I)), V([1, 1], H_B))
    add("order_case1_desc", "pfnOrderBy", Ls(V(rng.integers(0, 40, 5000).astype(np.int32), H_I), V(rng.integers(0, 20, 5000).astype(np.int32), H_I)), V([0, 0], H_B))
    k2 = rng.integers(0, 200, 8000).astype(np.int64)
    s2 = rng.integers(0, 2 ** 20, 8000).astype(np.int32)
    add("order_list_li_asc", "pfnOrderBy", Ls(V(k2, H_L), V(s2, H_I)), V([1, 1], H_B))
    add("order_list_li_mixed", "pfnOrderBy", Ls(V(k2, H_L), V(s2, H_I)), V([1, 0], H_B))
    add("order_list_li_desc", "pfnOrderBy", Ls(V(k2, H_L), V(s2, H_I)), V([0, 1], H_B))
    add("order_list_sorted_desc", "pfnOrderBy", Ls(V(np.sort(k2), H_L), V(s2, H_I)), V([0, 1], H_B))
    add("order_list_3col", "pfnOrderBy", Ls(V(rng.integers(0, 5, 3000).astype(np.int32), H_I), V(rng.integers(0, 5, 3000).astype(np.int64), H_L),
                                            V(rng.integers(0, 50, 3000).astype(np.int32), H_I)), V([1, 0, 1], H_B))
    add("order_f64", "pfnOrderBy", V(np.round(rng.standard_normal(3000), 1), H_E), V([1], H_B))
    add("order_char", "pfnOrderBy", V(rng.integers(0, 100, 3000).astype(np.int8), H_C), V([1], H_B))
    add("order_char_small", "pfnOrderBy", V([5, 3, 9, 3, 1], H_C), V([1], H_B))

    # ---- segmented reductions through each_right/each/raze (h_primitive.cc:1818-1904, 935-955)
    gk = rng.integers(0, 40, 5000).astype(np.int32)
    cases.append(dict(name="group_sum_chain", fn="@chain_group_agg", args=[V(gk, H_I), V(rng.uniform(0, 1e5, 5000), H_E)],
                      tol=1e-12, canonical=False, error=0))
    cases.append(dict(name="group_sum_chain_i32", fn="@chain_group_agg", args=[V(gk, H_I), V(rng.integers(-1000, 1000, 5000).astype(np.int32), H_I)],
                      tol=0.0, canonical=False, error=0))
    # ---- multi-column join_index (h_primitive.cc:2094-2110; joinOtherColumns h_system.cc:846-853)
    nb, npr = 3000, 9000
    bk = rng.integers(0, 2000, nb).astype(np.int32)                 # repeated keys: several pairs per probe row
    pk2 = rng.integers(0, 2000, npr).astype(np.int32)
    ba, pa = rng.integers(0, 50, nb).astype(np.int32), rng.integers(0, 50, npr).astype(np.int32)
    bd, pd = np.round(rng.standard_normal(nb), 1), np.round(rng.standard_normal(npr), 1)
    bl, pl = rng.integers(0, 30, nb).astype(np.int64), rng.integers(0, 30, npr).astype(np.int64)
    for ops, tag in [(["eq", "lt"], "eq_lt"), (["geq", "eq"], "geq_eq"), (["eq", "neq"], "eq_neq"), (["eq", "leq"], "eq_leq"),
                     (["eq", "gt"], "eq_gt"), (["eq", "eq"], "eq_eq")]:
        add(f"join_multi_{tag}", "pfnJoinIndex", Ls(V(bk, H_I), V(ba, H_I)), Ls(V(pk2, H_I), V(pa, H_I)), ("syms", ops))
    add("join_multi_f64", "pfnJoinIndex", Ls(V(bk, H_I), V(bd, H_E)), Ls(V(pk2, H_I), V(pd, H_E)), ("syms", ["eq", "lt"]))
    add("join_multi_mixed", "pfnJoinIndex", Ls(V(bk, H_I), V(bl, H_L), V(bd, H_E)),
        Ls(V(pk2, H_I), V(pa, H_I), V(pd.astype(np.float32), H_F)), ("syms", ["eq", "geq", "neq"]))
    add("join_multi_small_build", "pfnJoinIndex", Ls(V([4, 7, 4], H_I), V([1, 2, 3], H_I)),
        Ls(V(rng.integers(0, 9, 200).astype(np.int32), H_I), V(rng.integers(0, 4, 200).astype(np.int32), H_I)), ("syms", ["eq", "lt"]))
    add("join_multi_len_mismatch", "pfnJoinIndex", Ls(V(bk, H_I), V(ba, H_I)), Ls(V(pk2, H_I)), ("syms", ["eq", "lt"]), error=5)

    # ---- index_of on dates and symbols: hashed as ints, first occurrence (h_libs.h:25-31)
    dd = np.sort(rng.integers(9000, 9400, 3000)).astype(np.int32)      # sorted with repeats
    add("index_of_date", "pfnIndexOf", V(dd, H_D), V(rng.integers(8990, 9410, 4000).astype(np.int32), H_D))
    names = [f"s{i}" for i in range(40)]
    add("index_of_sym", "pfnIndexOf", ("syms", [names[i] for i in rng.integers(0, 30, 200)]),
        ("syms", [names[i] for i in rng.integers(0, 40, 300)]))
    add("index_of_date_vs_int", "pfnIndexOf", V(dd, H_D), V([9100], H_I), error=6)
    # strictly increasing keys (bucketed search on the GPU): skewed gaps, negatives, extremes
    sk = np.concatenate([np.arange(-3000, 2000, 3), [10 ** 12, 10 ** 12 + 5, 2 ** 62]]).astype(np.int64)
    probe = np.concatenate([rng.integers(-3100, 2100, 3000), [10 ** 12, 10 ** 12 + 1, 2 ** 62, -2 ** 63, 2 ** 63 - 1]])
    add("index_of_strict_skewed", "pfnIndexOf", V(sk, H_L), V(probe.astype(np.int64), H_L))
    si = np.unique(rng.integers(-2 ** 31, 2 ** 31 - 1, 5000)).astype(np.int32)
    add("index_of_strict_i32", "pfnIndexOf", V(si, H_I),
        V(np.concatenate([si[rng.integers(0, si.size, 2000)], rng.integers(-2 ** 31, 2 ** 31 - 1, 500)]).astype(np.int64), H_L))

    # ---- enum / foreign-key path (pfnEnum h_primitive.cc:2198-2222, pfnFetch/Keys/Values :191-225):
    #      chain outputs are values, fetch, keys, len, @index(key-side mask, values),
    #      the indices kept by a mask over the foreign keys and the key column gathered
    #      through them (the pattern of the reference's hand-written q5 plan)
    pk = rng.permutation(20000).astype(np.int32)                      # unsorted primary key: hash
    fk = pk[rng.integers(0, 20000, 50000)]
    cases.append(dict(name="enum_hash_i32", fn="@chain_enum", tol=0.0, canonical=False, error=0,
                      args=[V(pk, H_I), V(fk, H_I), V(rng.random(50000) < 0.3, H_B), V(rng.random(20000) < 0.5, H_B)]))
    pks = np.arange(1, 30001, dtype=np.int64) * 4                    # sorted primary key: binary search
    fks = pks[rng.integers(0, 30000, 60000)]
    cases.append(dict(name="enum_sorted_i64", fn="@chain_enum", tol=0.0, canonical=False, error=0,
                      args=[V(pks, H_L), V(fks, H_L), V(rng.random(60000) < 0.05, H_B), V(rng.random(30000) < 0.2, H_B)]))
    cases.append(dict(name="enum_promote", fn="@chain_enum", tol=0.0, canonical=False, error=0,
                      args=[V(pk.astype(np.int64), H_L), V(fk[:5000], H_I), V(rng.random(5000) < 0.5, H_B), V(rng.random(20000) < 0.5, H_B)]))
    dk = rng.permutation(np.arange(8000, 9000)).astype(np.int32)
    cases.append(dict(name="enum_date", fn="@chain_enum", tol=0.0, canonical=False, error=0,
                      args=[V(dk, H_D), V(dk[rng.integers(0, 1000, 3000)], H_D), V(rng.random(3000) < 0.5, H_B), V(rng.random(1000) < 0.5, H_B)]))
    cases.append(dict(name="enum_one", fn="@chain_enum", tol=0.0, canonical=False, error=0,
                      args=[V([5, 9, 2], H_I), V([2], H_I), V([True], H_B), V([True, False, True], H_B)]))
    cases.append(dict(name="enum_keep_one", fn="@chain_enum", tol=0.0, canonical=False, error=0,
                      args=[V([5, 9, 2], H_I), V([2, 5, 9, 9], H_I), V([False, False, True, False], H_B), V([True, False, True], H_B)]))
    add("enum_missing_key", "pfnEnum", V(pk, H_I), V(np.append(fk[:1000], 20001).astype(np.int32), H_I), error=10)
    add("enum_empty_key", "pfnEnum", V(np.zeros(0, np.int32), H_I), V([3], H_I), error=10)
    add("enum_type", "pfnEnum", V(pk, H_I), V(np.zeros(3, np.int32), H_D), error=6)

    # ---- @index_of / @enum on lists of columns (lib_index_of_G h_libs.cc:370-373, compareTuple h_system.cc:567-589)
    ka = rng.integers(0, 40, 3000).astype(np.int32)
    kb = rng.integers(-5, 25, 3000).astype(np.int64)
    qa = rng.integers(0, 45, 4000).astype(np.int32)
    qb = rng.integers(-8, 28, 4000).astype(np.int64)
    add("index_of_list_il", "pfnIndexOf", Ls(V(ka, H_I), V(kb, H_L)), Ls(V(qa, H_I), V(qb, H_L)))
    add("index_of_list_3", "pfnIndexOf", Ls(V(ka.astype(np.int16), H_H), V(kb.astype(np.int8), H_J), V(ka, H_I)),
        Ls(V(qa.astype(np.int16), H_H), V(qb.astype(np.int8), H_J), V(qa, H_I)))
    add("index_of_list_types", "pfnIndexOf", Ls(V(ka, H_I), V(kb, H_L)), Ls(V(qa.astype(np.int64), H_L), V(qb, H_L)))
    add("index_of_list_one", "pfnIndexOf", Ls(V(ka, H_I)), Ls(V(qa, H_I)))
    add("index_of_list_ncols", "pfnIndexOf", Ls(V(ka, H_I), V(kb, H_L)), Ls(V(qa, H_I)), error=1)
    add("index_of_list_ragged", "pfnIndexOf", Ls(V(ka, H_I), V(kb[:10], H_L)), Ls(V(qa, H_I), V(qb, H_L)), error=5)
    pairs = np.unique(np.stack([ka, kb], 1), axis=0)
    pick = pairs[rng.integers(0, len(pairs), 5000)]
    cases.append(dict(name="enum_list", fn="@chain_enum", tol=0.0, canonical=False, error=0,
                      args=[Ls(V(pairs[:, 0].astype(np.int32), H_I), V(pairs[:, 1], H_L)),
                            Ls(V(pick[:, 0].astype(np.int32), H_I), V(pick[:, 1], H_L)),
                            V(rng.random(5000) < 0.5, H_B), V(rng.random(len(pairs)) < 0.5, H_B)]))
    add("enum_list_missing", "pfnEnum", Ls(V(pairs[:, 0].astype(np.int32), H_I), V(pairs[:, 1], H_L)),
        Ls(V([999], H_I), V([0], H_L)), error=10)

    # ---- symbol compares (compareSymbol h_symbol.cc:241-243 under COMPFN h_primitive.cc:1068-1071)
    words = ["MAIL", "AIR", "REG AIR", "SHIP", "TRUCK", "RAIL", "FOB", "", "AIRMAIL", "air", "A", "MAIL "]
    sa = [words[i] for i in rng.integers(0, len(words), 400)]
    sb = [words[i] for i in rng.integers(0, len(words), 400)]
    for op in ["pfnLt", "pfnLeq", "pfnGt", "pfnGeq", "pfnEq", "pfnNeq"]:
        add(f"sym_{op[3:].lower()}_vv", op, ("syms", sa), ("syms", sb))
        add(f"sym_{op[3:].lower()}_vs", op, ("syms", sa), ("sym", "RAIL"))
        add(f"sym_{op[3:].lower()}_sv", op, ("sym", "AIR"), ("syms", sb))

    # ---- @like (pfnLike h_primitive.cc:1670-1758; genLikeString h_system.cc:319-334; PCRE2 anchored)
    letters = np.frombuffer(b"abcdefghijklmnopqrstuvwxyz      .", np.uint8)
    comments = []
    for k in range(600):
        n = int(rng.integers(0, 40))
        t = bytes(letters[rng.integers(0, len(letters), n)])
        if k % 7 == 0:
            t = t[:n // 2] + b"special" + t[n // 2:] + b"requests"
        if k % 11 == 0:
            t = b"PROMO " + t
        comments.append(t)
    comments += [b"", b"\n", b"abc", b"abc\n", b"ab\nc", b"a.c", b"abc.", b"a\\b", b"50%", b"special requests",
                 b"xspecialyrequestsz\n", b"\xe9t\xe9", b"a_c", b"aXc"]
    pats = ["%special%requests%", "PROMO%", "%requests", "_b%", "a.c", "a_c", "%", "", "abc", "%.%", "a\\b",
            "50%", "%s%s%s%", "__", "%\n%", "\xe9%"]
    for i, pat in enumerate(pats):
        if not pat:  # the reference's empty pattern reaches PCRE2 as NULL (crash); tested elsewhere
            continue
        pb = pat.encode("latin-1")
        add(f"like_str_{i}", "pfnLike", ("strs", comments), ("strs", [pb]))
    syms = ["MAIL", "AIR", "REG AIR", "SHIP", "TRUCK", "RAIL", "FOB", "AIRMAIL", "PROMO BRASS", "LARGE BRASS", "STANDARD"]
    col = [syms[i] for i in rng.integers(0, len(syms), 500)]
    for i, pat in enumerate(["%AIR%", "%BRASS", "PROMO%", "_A%", "%", "SHIP", "M__L"]):
        add(f"like_sym_{i}", "pfnLike", ("syms", col), ("sym", pat))
        add(f"like_sym_str_{i}", "pfnLike", ("syms", col), ("strs", [pat.encode()]))
    add("like_chars", "pfnLike", ("chars", b"forest green"), ("strs", [b"%green"]))
    add("like_chars_pat", "pfnLike", ("strs", [b"a", b"b", b"", b"ab"]), ("chars", b"_"))
    add("like_domain", "pfnLike", V([1, 2], H_I), ("strs", [b"%"]), error=1)
    add("like_length", "pfnLike", ("strs", [b"a", b"b", b"c"]), ("strs", [b"a", b"b"]), error=5)
    add("enum_list_len", "pfnEnum", Ls(V(pk[:10], H_I), V(pk[:10], H_I)), Ls(V(fk[:10], H_I)), error=1)

    # ---- the reference's quicksort paths (lib_quicksort_other h_libs.cc:409-442, lib_quicksort_list
    #      :637-697, lib_order_by_sorted :604-617): keys other than i32/i64/char, alone and in lists,
    #      with many ties, at 100K+ rows (own generator, so the cases above keep their inputs)
    q = np.random.default_rng(20261204)
    N = 120_000
    f_ties = np.round(q.standard_normal(N), 1)                            # ~80 distinct values
    f_ties[q.random(N) < 0.05] = -0.0                                     # -0.0 ties +0.0
    add("qs_order_f64_asc_120k", "pfnOrderBy", V(f_ties, H_E), V([1], H_B))
    add("qs_order_f64_desc_120k", "pfnOrderBy", V(f_ties, H_E), V([0], H_B))
    add("qs_group_f64_120k", "pfnGroup", V(f_ties, H_E))
    add("qs_order_f32_120k", "pfnOrderBy", V(f_ties.astype(np.float32), H_F), V([1], H_B))
    j3 = q.integers(-1, 2, N).astype(np.int8)
    add("qs_order_i8_120k", "pfnOrderBy", V(j3, H_J), V([1], H_B))
    add("qs_order_i16_desc_120k", "pfnOrderBy", V(q.integers(-300, 300, N).astype(np.int16), H_H), V([0], H_B))
    add("qs_order_bool_120k", "pfnOrderBy", V(q.random(N) < 0.5, H_B), V([1], H_B))
    add("qs_group_bool_120k", "pfnGroup", V(q.random(N) < 0.3, H_B))
    add("qs_group_i16_120k", "pfnGroup", V(q.integers(0, 40, N).astype(np.int16), H_H))
    add("qs_order_date_120k", "pfnOrderBy", V(q.integers(8000, 8400, N).astype(np.int32), H_D), V([1], H_B))
    add("qs_group_date_120k", "pfnGroup", V(q.integers(8000, 8100, N).astype(np.int32), H_D))
    add("qs_group_list_jj_120k", "pfnGroup", Ls(V(q.integers(0, 3, N).astype(np.int8), H_J), V(q.integers(0, 2, N).astype(np.int8), H_J)))
    add("qs_group_list_ej_120k", "pfnGroup", Ls(V(np.round(q.standard_normal(N), 0), H_E), V(q.integers(0, 4, N).astype(np.int8), H_J)))
    add("qs_group_list_il_e", "pfnGroup", Ls(V(q.integers(0, 30, N).astype(np.int32), H_I), V(np.round(q.standard_normal(N), 0), H_E)))
    add("qs_group_list_one_neg_i32", "pfnGroup", Ls(V(q.integers(-50, 50, 20000).astype(np.int32), H_I)))
    add("qs_group_list_one_f64", "pfnGroup", Ls(V(np.round(q.standard_normal(20000), 1), H_E)))
    ek, ik = np.round(q.standard_normal(N), 0), q.integers(0, 50, N).astype(np.int32)
    add("qs_order_list_ei_asc", "pfnOrderBy", Ls(V(ek, H_E), V(ik, H_I)), V([1, 1], H_B))
    add("qs_order_list_ei_mixed", "pfnOrderBy", Ls(V(ek, H_E), V(ik, H_I)), V([0, 1], H_B))
    add("qs_order_list_ie_mixed", "pfnOrderBy", Ls(V(ik, H_I), V(ek, H_E)), V([1, 0], H_B))
    add("qs_order_list_jel", "pfnOrderBy", Ls(V(j3, H_J), V(ek, H_E), V(q.integers(0, 9, N).astype(np.int64), H_L)), V([1, 0, 1], H_B))
    add("qs_order_list_ci", "pfnOrderBy", Ls(V(q.integers(65, 70, N).astype(np.int8), H_C), V(ik, H_I)), V([1, 1], H_B))
    add("qs_order_list_ic_small_runs", "pfnOrderBy", Ls(V(q.integers(0, 20000, 60000).astype(np.int32), H_I),
                                                     V(q.integers(65, 90, 60000).astype(np.int8), H_C)), V([1, 1], H_B))
    add("qs_order_list_dd", "pfnOrderBy", Ls(V(q.integers(8000, 8050, N).astype(np.int32), H_D), V(q.integers(0, 7, N).astype(np.int16), H_H)), V([0, 0], H_B))
    # ranges already in order: kept (ascending) or reversed (descending key whose values ascend)
    srt = np.sort(np.round(q.standard_normal(50000), 2))
    add("qs_order_list_sorted_e_desc", "pfnOrderBy", Ls(V(srt, H_E), V(q.integers(0, 3, 50000).astype(np.int8), H_J)), V([0, 1], H_B))
    add("qs_order_list_runs_sorted", "pfnOrderBy", Ls(V(np.repeat(np.arange(500), 100).astype(np.int32), H_I),
                                                   V(np.tile(np.round(np.linspace(-3, 3, 100), 1), 500), H_E)), V([1, 0], H_B))
    # deep recursion: the first-element pivot on ordered keys peels one element per level
    add("qs_order_f64_sorted_3k", "pfnOrderBy", V(np.sort(q.standard_normal(3000)), H_E), V([1], H_B))
    add("qs_order_f64_reverse_3k", "pfnOrderBy", V(np.sort(q.standard_normal(3000))[::-1].copy(), H_E), V([1], H_B))
    add("qs_group_f64_tiny", "pfnGroup", V([2.0, -0.0, 0.0, 2.0, 1.5], H_E))
    add("qs_order_f64_one", "pfnOrderBy", V([3.5], H_E), V([0], H_B))
    add("qs_order_f64_empty", "pfnOrderBy", V(np.zeros(0), H_E), V([1], H_B))
    return cases
