"""bench.py runs only on a GPU machine; this CPU check catches the mistakes that
would only surface there: names a function reads but never binds (neither
locally, nor at module level, nor as a builtin), and the JSON keys the
default line must carry."""
import ast
import builtins
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _module():
    with open(os.path.join(ROOT, "bench.py")) as f:
        return ast.parse(f.read())


def test_no_unbound_names_in_bench():
    tree = _module()
    top = set()
    for n in tree.body:
        if isinstance(n, (ast.FunctionDef, ast.ClassDef)):
            top.add(n.name)
        elif isinstance(n, ast.Assign):
            top |= {t.id for t in n.targets if isinstance(t, ast.Name)}
        elif isinstance(n, (ast.Import, ast.ImportFrom)):
            top |= {(a.asname or a.name).split(".")[0] for a in n.names}
    missing = []
    for fn in (n for n in tree.body if isinstance(n, ast.FunctionDef)):
        bound = {a.arg for a in fn.args.args} | {a.arg for a in fn.args.kwonlyargs}
        for node in ast.walk(fn):
            if isinstance(node, ast.Name) and isinstance(node.ctx, (ast.Store, ast.Del)):
                bound.add(node.id)
            elif isinstance(node, (ast.Import, ast.ImportFrom)):
                bound |= {(a.asname or a.name).split(".")[0] for a in node.names}
            elif isinstance(node, (ast.FunctionDef, ast.Lambda)) and node is not fn:
                bound |= {a.arg for a in node.args.args}
                if isinstance(node, ast.FunctionDef):
                    bound.add(node.name)
            elif isinstance(node, ast.ExceptHandler) and node.name:
                bound.add(node.name)
        for node in ast.walk(fn):
            if isinstance(node, ast.Name) and isinstance(node.ctx, ast.Load):
                if node.id not in bound and node.id not in top and not hasattr(builtins, node.id):
                    missing.append(f"{fn.name}:{node.lineno}:{node.id}")
    assert not missing, missing


def test_default_line_keys_present():
    src = open(os.path.join(ROOT, "bench.py")).read()
    tree = ast.parse(src)
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "run_flow")
    keys = {k.value for node in ast.walk(fn) if isinstance(node, ast.Dict) for k in node.keys
            if isinstance(k, ast.Constant)}
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "gpu_launches", "clocks"):
        assert k in keys, k
    assert "cpu_baseline" in src
