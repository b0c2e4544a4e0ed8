#!/usr/bin/env python3
"""Extract the known-answer cases of LUE's routing-operation unit tests into JSON.

This script reads the reference's Boost.Test sources as TEXT (nothing is compiled or run) and
writes ``reference_cases.json`` beside itself.  The JSON is committed; the tests only read the
JSON, so the reference tree is needed only when regenerating it:

    python tests/golden/extract_reference_cases.py --reference <root of the reference project>

Sources read (paths within the reference project):

- source/framework/algorithm/test/flow_accumulation.hpp       shared 9x9 / 3x3 fixture shapes, D8 names
- source/framework/algorithm/test/flow_accumulation.cpp.in    merging_streams, spiral_in, pcraster example, ...
- source/framework/algorithm/test/accu_test.cpp
- source/framework/algorithm/test/accu_threshold_test.cpp
- source/framework/algorithm/test/accu_fraction_test.cpp
- source/framework/algorithm/test/kinematic_wave_test.cpp
- source/framework/algorithm/test/inflow_count_test.cpp
- source/framework/algorithm/test/d8_flow_direction_test.cpp
- source/framework/algorithm/test/accu_capacity_test.cpp, accu_trigger_test.cpp
- source/framework/algorithm/test/upstream_test.cpp, downstream_test.cpp, downstream_distance_test.cpp
- source/framework/algorithm/test/accu_info_test.cpp

Each ``create_partitioned_array(shape, partition_shape, {{partition}, ...})`` literal lists its
partitions in row-major partition order, each partition's cells row-major.  Partition extents follow
the reference's domain decomposition (``source/framework/core/include/lue/framework/core/
domain_decomposition.hpp:90-175``): ``floor(shape / partition_shape)`` partitions per dimension, the
last one absorbing the remainder.  The assembled rasters are stored row-major for the whole array;
NaN (the float no-data value) is stored as JSON ``null``.
"""
import argparse
import json
import math
import os
import re
import sys

TEST_DIR = "source/framework/algorithm/test"
# where the reference's sources are mounted when the fixture is regenerated: --reference, or LUE_REFERENCE
DEFAULT_REFERENCE = os.environ.get("LUE_REFERENCE")

# D8 keypad codes, source/framework/algorithm/include/lue/framework/algorithm/flow_direction.hpp:7-35
D8 = {"nw": 7, "n": 8, "ne": 9, "w": 4, "p": 5, "e": 6, "sw": 1, "s": 2, "se": 3}
U8_NO_DATA = 255
# accu_info cell classes, source/framework/algorithm/include/lue/framework/algorithm/accu_info.hpp:22-63
CELL_CLASSES = {"ridge_cell": 11, "intra_partition_stream_cell": 12, "partition_output_cell": 13,
                "partition_input_cell": 14, "partition_input_output_cell": 15, "inter_partition_stream_cell": 16,
                "sink_cell": 17, "confluence_cell": 18}


def strip_comments(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    return text


def matching(text, start, open_ch, close_ch):
    """Index of the bracket closing the one at text[start]."""
    depth = 0
    for i in range(start, len(text)):
        c = text[i]
        if c == open_ch:
            depth += 1
        elif c == close_ch:
            depth -= 1
            if depth == 0:
                return i
    raise ValueError("unbalanced")


def split_top(text, sep=","):
    """Split on separators at bracket depth 0 (templates are tracked only inside create_* calls)."""
    parts, depth, cur = [], 0, []
    for c in text:
        if c in "({[":
            depth += 1
        elif c in ")}]":
            depth -= 1
        if c == sep and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(c)
    tail = "".join(cur)
    if tail.strip():
        parts.append(tail)
    return [p.strip() for p in parts]


def split_statements(body):
    stmts, depth, cur = [], 0, []
    for c in body:
        if c in "({[":
            depth += 1
        elif c in ")}]":
            depth -= 1
        if c == ";" and depth == 0:
            stmts.append("".join(cur).strip())
            cur = []
        else:
            cur.append(c)
    return [s for s in stmts if s]


def test_cases(text):
    """Yield (name, line, body) for every BOOST_AUTO_TEST_CASE."""
    for m in re.finditer(r"BOOST_AUTO_TEST_CASE\((\w+)\)", text):
        brace = text.index("{", m.end())
        end = matching(text, brace, "{", "}")
        yield m.group(1), text.count("\n", 0, m.start()) + 1, text[brace + 1:end]


def partition_extents(extent, pextent):
    n = max(extent // pextent, 1)
    sizes = [pextent] * n
    sizes[-1] = extent - pextent * (n - 1)
    return sizes


def assemble(shape, pshape, partitions):
    rows, cols = shape
    rsizes = partition_extents(rows, pshape[0])
    csizes = partition_extents(cols, pshape[1])
    if len(partitions) != len(rsizes) * len(csizes):
        raise ValueError(f"{len(partitions)} partitions for grid {len(rsizes)}x{len(csizes)}")
    out = [[None] * cols for _ in range(rows)]
    k = 0
    r0 = 0
    for pr in rsizes:
        c0 = 0
        for pc in csizes:
            part = partitions[k]
            if len(part) != pr * pc:
                raise ValueError(f"partition {k} has {len(part)} cells, want {pr * pc}")
            for i in range(pr):
                for j in range(pc):
                    out[r0 + i][c0 + j] = part[i * pc + j]
            k += 1
            c0 += pc
        r0 += pr
    return out


class Env:
    """Symbol table of one scope: D8 names, no-data aliases, shapes, scalars and arrays."""

    def __init__(self, parent=None):
        self.parent = parent
        self.values = {}
        self.shapes = {}
        self.arrays = {}

    def lookup(self, table, name):
        env = self
        while env is not None:
            t = getattr(env, table)
            if name in t:
                return t[name]
            env = env.parent
        raise KeyError(name)


def elem_kind(type_text):
    """'u8' for flow directions and counts, 'f' for material."""
    t = type_text
    if "FlowDirection" in t or "CountElement" in t or "InflowCount" in t or "uint8" in t or "CellClass" in t:
        return "u8"
    return "f"


def eval_scalar(expr, env, kind="f"):
    e = expr.strip()
    e = re.sub(r"^lue::test::", "", e)
    m = re.fullmatch(r"lue::policy::no_data_value<([\w:]+)>", e)
    if m:
        return U8_NO_DATA if elem_kind(m.group(1)) == "u8" else math.nan
    m = re.fullmatch(r"(\w+)\{(.*)\}", e)  # MaterialElement{0}
    if m and not m.group(1)[0].isdigit():
        return eval_scalar(m.group(2), env, kind)
    try:
        v = float(e.rstrip("f"))
        return int(v) if kind == "u8" else v
    except ValueError:
        pass
    return env.lookup("values", e)


def eval_shape(expr, env):
    e = expr.strip()
    e = re.sub(r"^lue::test::", "", e)
    m = re.fullmatch(r"\{?\{?\s*(\d+)\s*,\s*(\d+)\s*\}?\}?", e)
    if m:
        return (int(m.group(1)), int(m.group(2)))
    m = re.fullmatch(r"(\w+)\.shape\(\)", e)
    if m:
        arr = env.lookup("arrays", m.group(1))
        return (len(arr["data"]), len(arr["data"][0]))
    return env.lookup("shapes", e)


def fill(shape, value):
    return [[value] * shape[1] for _ in range(shape[0])]


def eval_array(expr, env, fixtures):
    """Evaluate an array-valued expression to {'kind', 'data', 'partition_shape'}."""
    e = expr.strip()
    m = re.match(r"(?:lue::)?(?:test::)?create_partitioned_array\s*<(.*?)>\s*\(", e, flags=re.S)
    if m:
        type_text = m.group(1)
        # the template argument can itself contain '<...>'; find the '(' that opens the call
        open_paren = e.index("(", m.start() + len("create_partitioned_array"))
        # move open_paren past the complete template argument list
        lt = e.index("<", m.start())
        depth = 0
        for i in range(lt, len(e)):
            if e[i] == "<":
                depth += 1
            elif e[i] == ">":
                depth -= 1
                if depth == 0:
                    open_paren = e.index("(", i)
                    type_text = e[lt + 1:i]
                    break
        close = matching(e, open_paren, "(", ")")
        args = split_top(e[open_paren + 1:close])
        kind = elem_kind(type_text)
        shape = eval_shape(args[0], env)
        pshape = eval_shape(args[1], env)
        if args[2].startswith("{"):
            inner = args[2].strip()[1:-1]
            partitions = []
            for part in split_top(inner):
                if not part:
                    continue
                cells = [eval_scalar(c, env, kind) for c in split_top(part.strip()[1:-1]) if c]
                partitions.append(cells)
            data = assemble(shape, pshape, partitions)
        else:
            data = fill(shape, eval_scalar(args[2], env, kind))
        return {"kind": kind, "data": data, "partition_shape": list(pshape)}
    m = re.fullmatch(r"lue::test::(ones|zeros|no_data)<(\w+)>\(\)", e)
    if m:
        kind = elem_kind(m.group(2))
        value = {"ones": 1, "zeros": 0}.get(m.group(1))
        if value is None:
            value = U8_NO_DATA if kind == "u8" else math.nan
        return {"kind": kind, "data": fill((9, 9), value), "partition_shape": [3, 3]}
    m = re.fullmatch(r"lue::test::filled(?:<(\w+)>)?\((.*)\)", e, flags=re.S)
    if m:
        arg = m.group(2).strip()
        if m.group(1):
            kind = elem_kind(m.group(1))
        elif "no_data_value" in arg:
            kind = elem_kind(re.search(r"<(\w+)>", arg).group(1))
        else:
            kind = "u8" if re.sub(r"^lue::test::", "", arg) in D8 else "f"
        return {"kind": kind, "data": fill((9, 9), eval_scalar(arg, env, kind)),
                "partition_shape": [3, 3]}
    m = re.fullmatch(r"lue::test::(\w+)\(\)", e)
    if m and m.group(1) in fixtures:
        return fixtures[m.group(1)]
    raise ValueError(f"cannot evaluate array expression: {e[:120]}")


def base_env():
    env = Env()
    for k, v in D8.items():
        env.values[k] = v
    env.values["nd"] = U8_NO_DATA
    env.shapes["array_shape"] = (9, 9)
    env.shapes["partition_shape"] = (3, 3)
    return env


def process_statements(stmts, env, fixtures, on_call):
    for s in stmts:
        s1 = " ".join(s.split())
        # shape declarations
        m = re.match(r".*?\b(array_shape|partition_shape)\s*(?:\{(.*)\}|=\s*(.*))$", s1)
        if m and ("Shape" in s1 or "auto" in s1) and "create_partitioned_array" not in s1:
            env.shapes[m.group(1)] = eval_shape(m.group(2) or m.group(3), env)
            continue
        # aliases: auto const n = lue::test::n / auto const x{no_data_value<...>}
        m = re.match(r"auto const (\w+)\s*(?:=\s*|\{)(lue::test::\w+|lue::policy::no_data_value<[\w:]+>)\}?$", s1)
        if m:
            env.values[m.group(1)] = eval_scalar(m.group(2), env, elem_kind(m.group(2)))
            continue
        # accu_info cell classes: auto const intra = lue::intra_partition_stream_cell
        m = re.match(r"auto const (\w+)\s*=\s*lue::(\w+_cell)$", s1)
        if m and m.group(2) in CELL_CLASSES:
            env.values[m.group(1)] = CELL_CLASSES[m.group(2)]
            continue
        # scalars
        m = re.match(r"lue::Scalar<\w+> const (\w+)\s*(?:=\s*(.*)|\{(.*)\})$", s1)
        if m:
            text = (m.group(2) or m.group(3) or "").strip()
            if text:  # default-constructed scalars (overload-only cases) carry no value
                env.values[m.group(1)] = eval_scalar(text, env)
            continue
        m = re.match(r"(?:auto const|auto|\w+ const|lue::PartitionedArray<[^=]*?>(?: const)?) (\w+)\s*=\s*(lue::.*)$", s,
                     flags=re.S)
        if m and ("create_partitioned_array" in m.group(2) or re.match(r"lue::test::\w+(<\w+>)?\(", m.group(2).strip())):
            env.arrays[m.group(1)] = eval_array(m.group(2), env, fixtures)
            continue
        on_call(s, env)


def parse_fixtures(text):
    """flow_accumulation.cpp.in: the shared flow-direction rasters (9x9 in 3x3, pcraster example 5x5)."""
    fixtures = {}
    env = base_env()
    for m in re.finditer(r"(?:FlowDirectionArray|auto)\s+(\w+)\(\)\s*(?:->\s*FlowDirectionArray\s*)?\{", text):
        name = m.group(1)
        brace = m.end() - 1
        end = matching(text, brace, "{", "}")
        body = text[brace + 1:end]
        local = Env(env)
        result = {}

        def on_call(s, e, result=result):
            if s.startswith("return"):
                result["array"] = eval_array(s[len("return"):], e, fixtures)

        process_statements(split_statements(body), local, fixtures, on_call)
        fixtures[name] = result["array"]
    return fixtures


OPS = ("accu_threshold", "accu_fraction", "kinematic_wave", "accu", "accu_capacity", "accu_trigger", "upstream",
       "downstream", "accu_info")


def extract_file(path, rel, fixtures, cases):
    text = strip_comments(open(path).read())
    file_env = base_env()
    # file-level shapes/aliases (inflow_count_test.cpp anonymous namespace)
    ns = re.search(r"namespace\s*\{(.*?)\}\s*(?=BOOST_AUTO_TEST_CASE)", text, flags=re.S)
    if ns:
        process_statements(split_statements(ns.group(1)), file_env, fixtures, lambda s, e: None)
    for name, line, body in test_cases(text):
        env = Env(file_env)
        calls = []

        def on_call(s, e, calls=calls):
            s1 = " ".join(s.split())
            m = re.search(r"value_policies::(\w+)(?:<[^>]*>)?\((.*)\)$", s1)
            if m and m.group(1) in OPS:
                lhs = s1[:m.start()]
                outs = re.findall(r"(\w+_we_got)", lhs)
                calls.append({"op": m.group(1), "args": split_top(m.group(2)), "outs": outs})
                return
            m = re.search(r"detail::iterate_to_new_discharge<\w+>\((.*)\)\}?$", s1)
            if m:
                calls.append({"op": "iterate_to_new_discharge",
                              "args": [float(a) for a in split_top(m.group(1))]})
                return
            m = re.search(r"outflow_we_want\{(.*)\}$", s1)
            if m and calls and calls[-1]["op"] == "iterate_to_new_discharge":
                v = m.group(1).strip()
                calls[-1]["expected"] = 0.0 if v == "0" else (
                    2.2250738585072014e-308 if "numeric_limits" in v else float(v))
                return
            m = re.match(r"test_inflow_count\((.*)\)$", s, flags=re.S)
            if m:
                text = m.group(1)
                pol = re.match(r"\s*lue::policy::inflow_count::(\w+)<[^>]*>\{\}\s*,", text)
                value_policies = bool(pol) and pol.group(1) == "DefaultValuePolicies"
                if pol:
                    text = text[pol.end():]
                args = split_top(text)
                arrs = [e.lookup("arrays", a) if re.fullmatch(r"\w+", a) else eval_array(a, e, fixtures)
                        for a in args]
                calls.append({"op": "inflow_count", "fd": arrs[0], "want": arrs[1],
                              "no_data_policy": value_policies})
                return
            m = re.search(r"check_arrays_are_(equal|close)\((\w+), (\w+)\)", s1)
            if m:
                calls.append({"op": "check", "how": m.group(1), "got": m.group(2), "want": m.group(3)})
                return
            if "all(outflow_we_got > " in s1:
                calls.append({"op": "check_all_positive"})

        # scalar solves sit in nested blocks: take each call with the expectation that follows it
        for m in re.finditer(r"iterate_to_new_discharge<\w+>\(([^)]*)\)\}.*?outflow_we_want\{([^}]*)\}",
                             body, flags=re.S):
            want = m.group(2).strip()
            calls.append({"op": "iterate_to_new_discharge",
                          "args": [float(a) for a in split_top(m.group(1))],
                          "expected": 2.2250738585072014e-308 if "numeric_limits" in want else float(want)})
        if any(c["op"] == "iterate_to_new_discharge" for c in calls):
            emit_cases(rel, name, line, env, calls, cases)
            continue
        process_statements(split_statements(body), env, fixtures, on_call)
        emit_cases(rel, name, line, env, calls, cases)


def arr(a):
    return [[None if (isinstance(v, float) and math.isnan(v)) else v for v in row] for row in a["data"]]


def arg_value(env, name):
    try:
        a = env.lookup("arrays", name)
        return {"raster": arr(a)}
    except KeyError:
        v = env.lookup("values", name)
        return {"scalar": None if (isinstance(v, float) and math.isnan(v)) else v}


def emit_cases(rel, name, line, env, calls, cases):
    base = {"file": rel, "line": line, "name": name}
    for c in calls:
        if c["op"] == "inflow_count":
            cases.append({**base, "op": "inflow_count", "no_data_policy": c["no_data_policy"],
                          "partition_shape": c["fd"]["partition_shape"],
                          "flow_direction": arr(c["fd"]), "expected": {"inflow_count": arr(c["want"])},
                          "compare": "equal"})
        elif c["op"] == "iterate_to_new_discharge":
            keys = ["upstream_discharge", "current_outflow", "lateral_inflow", "alpha", "beta",
                    "time_step_duration", "channel_length"]
            cases.append({**base, "op": "iterate_to_new_discharge", "args": dict(zip(keys, c["args"])),
                          "expected": c["expected"], "compare": "close_or_small_1e-6"})
        elif c["op"] in OPS:
            if not c["args"] or c["args"][0] != "flow_direction":
                continue
            try:
                fd = env.lookup("arrays", "flow_direction")
            except KeyError:
                continue  # overload-only case with default-constructed arrays
            checks = [k for k in calls if k["op"] == "check"]
            expected = {}
            how = "equal"
            for k in checks:
                expected[k["got"]] = arr(env.lookup("arrays", k["want"]))
                how = k["how"]
            positive = any(k["op"] == "check_all_positive" for k in calls)
            if not expected and not positive:
                continue
            inputs = {a: arg_value(env, a) for a in c["args"][1:]}
            cases.append({**base, "op": c["op"], "partition_shape": fd["partition_shape"],
                          "flow_direction": arr(fd), "inputs": inputs, "outputs": c["outs"],
                          "expected": expected,
                          "compare": "all_positive" if positive and not expected else how})


def extract_d8(path, rel, fixtures, cases):
    """d8_flow_direction_test.cpp: pairs of (elevation, flow_direction_we_want) literals, in source
    order, for every case that checks them (barnes_2017 only warns, so it pins nothing)."""
    text = strip_comments(open(path).read())
    for name, line, body in test_cases(text):
        if "check_arrays_are_equal" not in body:
            continue
        env = Env(base_env())
        # aliases and shapes declared at the top of the case
        process_statements([st for st in split_statements(body) if "create_partitioned_array" not in st
                            and "d8_flow_direction<" not in st and not st.lstrip().startswith("{")],
                           env, fixtures, lambda st, e: None)
        env.values.setdefault("y", D8["p"])
        env.values["x"] = math.nan
        env.values["u"] = U8_NO_DATA
        arrays = []
        for m in re.finditer(r"(elevation|flow_direction_we_want)\s*=\s*lue::test::create_partitioned_array", body):
            start = m.start(0) + body[m.start(0):].index("lue::test::")
            close = matching(body, body.index("(", body.index(">", start)), "(", ")")
            arrays.append((m.group(1), eval_array(body[start:close + 1], env, fixtures)))
        for (k1, elev), (k2, want) in zip(arrays[0::2], arrays[1::2]):
            assert k1 == "elevation" and k2 == "flow_direction_we_want"
            cases.append({"file": rel, "line": line, "name": name, "op": "d8_flow_direction",
                          "partition_shape": elev["partition_shape"], "elevation": arr(elev),
                          "expected": {"flow_direction": [[int(v) for v in row] for row in want["data"]]},
                          "compare": "equal"})


def extract_downstream_distance(path, rel, fixtures, cases):
    """downstream_distance_test.cpp: a flow-direction literal, the cell size and the distances wanted
    (q stands for sqrt(2) * cell size)."""
    text = strip_comments(open(path).read())
    for name, line, body in test_cases(text):
        env = Env(base_env())
        m = re.search(r"cell_size\s*\{\s*([0-9.]+)\s*\}", body)
        if not m:
            continue
        cell = float(m.group(1))
        env.values["q"] = math.sqrt(2.0) * cell
        for st in split_statements(body):
            s1 = " ".join(st.split())
            mm = re.match(r".*?\b(array_shape|partition_shape)\s*\{(.*)\}$", s1)
            if mm and "Shape" in s1:
                env.shapes[mm.group(1)] = eval_shape(mm.group(2), env)
        arrays = {}
        for mm in re.finditer(r"(flow_direction|result_we_want)\s*=\s*lue::test::create_partitioned_array", body):
            start = mm.start(0) + body[mm.start(0):].index("lue::test::")
            close = matching(body, body.index("(", body.index(">", start)), "(", ")")
            kind_env = Env(env)
            arrays[mm.group(1)] = eval_array(body[start:close + 1], kind_env, fixtures)
        if set(arrays) != {"flow_direction", "result_we_want"}:
            continue
        cases.append({"file": rel, "line": line, "name": name, "op": "downstream_distance",
                      "partition_shape": arrays["flow_direction"]["partition_shape"],
                      "flow_direction": arr(arrays["flow_direction"]), "cell_size": cell,
                      "expected": {"distance": arr(arrays["result_we_want"])}, "compare": "close"})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=DEFAULT_REFERENCE,
                    help="root of the reference project's sources (default: $LUE_REFERENCE)")
    ap.add_argument("--out", default=os.path.join(os.path.dirname(__file__), "reference_cases.json"))
    a = ap.parse_args()
    if not a.reference:
        ap.error("give the reference project's root with --reference or LUE_REFERENCE")
    tdir = os.path.join(a.reference, TEST_DIR)
    fixtures = parse_fixtures(strip_comments(open(os.path.join(tdir, "flow_accumulation.cpp.in")).read()))
    cases = []
    for f in ("accu_test.cpp", "accu_threshold_test.cpp", "accu_fraction_test.cpp",
              "kinematic_wave_test.cpp", "inflow_count_test.cpp", "accu_capacity_test.cpp",
              "accu_trigger_test.cpp", "upstream_test.cpp", "downstream_test.cpp", "accu_info_test.cpp"):
        extract_file(os.path.join(tdir, f), f"{TEST_DIR}/{f}", fixtures, cases)
    extract_downstream_distance(os.path.join(tdir, "downstream_distance_test.cpp"),
                                f"{TEST_DIR}/downstream_distance_test.cpp", fixtures, cases)
    extract_d8(os.path.join(tdir, "d8_flow_direction_test.cpp"), f"{TEST_DIR}/d8_flow_direction_test.cpp",
               fixtures, cases)
    with open(a.out, "w") as fh:
        json.dump({"generated_by": "tests/golden/extract_reference_cases.py",
                   "source": "computationalgeography/lue " + TEST_DIR, "cases": cases}, fh, indent=None)
        fh.write("\n")
    by_op = {}
    for c in cases:
        by_op[c["op"]] = by_op.get(c["op"], 0) + 1
    print(f"{len(cases)} cases: {by_op}", file=sys.stderr)


if __name__ == "__main__":
    main()
