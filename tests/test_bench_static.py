"""Static checks of bench.py that need no GPU: every name a function reads is defined (a
parameter, a local, a module global, an import or a builtin), so that a workload path the CPU
suite cannot run does not fail on a stray name at the end of a GPU run."""
import ast
import builtins
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bound_names(fn):
    names = {a.arg for a in fn.args.args + fn.args.kwonlyargs + fn.args.posonlyargs}
    if fn.args.vararg:
        names.add(fn.args.vararg.arg)
    if fn.args.kwarg:
        names.add(fn.args.kwarg.arg)
    for node in ast.walk(fn):
        if isinstance(node, ast.Name) and isinstance(node.ctx, (ast.Store, ast.Del)):
            names.add(node.id)
        elif isinstance(node, (ast.FunctionDef, ast.AsyncFunctionDef, ast.ClassDef)) and node is not fn:
            names.add(node.name)
            if not isinstance(node, ast.ClassDef):
                names.update(a.arg for a in node.args.args + node.args.kwonlyargs)
        elif isinstance(node, ast.Lambda):
            names.update(a.arg for a in node.args.args)
        elif isinstance(node, (ast.Import, ast.ImportFrom)):
            names.update((a.asname or a.name).split(".")[0] for a in node.names)
        elif isinstance(node, ast.ExceptHandler) and node.name:
            names.add(node.name)
        elif isinstance(node, ast.comprehension):
            for t in ast.walk(node.target):
                if isinstance(t, ast.Name):
                    names.add(t.id)
    return names


def test_bench_functions_read_only_defined_names():
    tree = ast.parse(open(os.path.join(ROOT, "bench.py")).read())
    module_names = set(dir(builtins))
    for node in tree.body:
        if isinstance(node, (ast.FunctionDef, ast.ClassDef)):
            module_names.add(node.name)
        elif isinstance(node, (ast.Import, ast.ImportFrom)):
            module_names.update((a.asname or a.name).split(".")[0] for a in node.names)
        elif isinstance(node, (ast.Assign, ast.AnnAssign)):
            targets = node.targets if isinstance(node, ast.Assign) else [node.target]
            for t in targets:
                for n in ast.walk(t):
                    if isinstance(n, ast.Name):
                        module_names.add(n.id)
    enclosing = {}  # function -> the functions it is nested in (closures read their names)
    for outer in ast.walk(tree):
        if isinstance(outer, ast.FunctionDef):
            for inner in ast.walk(outer):
                if isinstance(inner, ast.FunctionDef) and inner is not outer:
                    enclosing.setdefault(inner, []).append(outer)
    missing = []
    for fn in ast.walk(tree):
        if not isinstance(fn, ast.FunctionDef):
            continue
        bound = _bound_names(fn) | module_names
        for outer in enclosing.get(fn, []):
            bound |= _bound_names(outer)
        for node in ast.walk(fn):
            if isinstance(node, ast.Name) and isinstance(node.ctx, ast.Load) and node.id not in bound:
                missing.append(f"{fn.name}:{node.lineno}: {node.id}")
    assert not missing, missing


def test_reference_arm_on_the_app_frame():
    """`bench.py --impl reference --workload app-solar-4444` runs on the CPU alone: the app's
    scene from the oracle's restatement of its generator, the literal walk, one JSON line."""
    import json
    import subprocess
    import sys

    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "app-solar-4444", "--steps", "1", "--warmup", "3"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["config"]["workload"] == "app-solar-4444" and d["config"]["bodies"] == 4444
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
