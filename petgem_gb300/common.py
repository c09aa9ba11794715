"""Params file, timers and rank-0 printing, mirroring petgem/common.py.

``InputParameters`` reads the same YAML params file and applies the same
consistency checks as petgem/common.py:137-361; where petgem prints and
calls ``exit(-1)`` this raises ``ParamsError``.  PyYAML is used when it is
installed; otherwise a parser for the YAML subset petgem's params files use
(nested block mappings, flow lists, scalars, comments) reads the file.
"""
import ast
import os
import sys
import time


class ParamsError(ValueError):
    """Inconsistent or missing parameter (petgem prints and exits instead)."""


# ----------------------------------------------------------------------------- YAML subset
def _scalar(tok):
    t = tok.strip()
    if t == "":
        return None
    if (t[0] == t[-1]) and t[0] in "'\"" and len(t) >= 2:
        return t[1:-1]
    low = t.lower()
    if low in ("true", "yes", "on"):
        return True
    if low in ("false", "no", "off"):
        return False
    if low in ("null", "none", "~"):
        return None
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(t)
    except ValueError:
        pass
    return t


def _flow(t):
    t = t.strip()
    if t.startswith("[") and t.endswith("]"):
        inner = t[1:-1].strip()
        if not inner:
            return []
        out, depth, cur = [], 0, ""
        for ch in inner:
            if ch == "," and depth == 0:
                out.append(_flow(cur))
                cur = ""
                continue
            depth += ch == "["
            depth -= ch == "]"
            cur += ch
        out.append(_flow(cur))
        return out
    return _scalar(t)


def _strip_comment(line):
    out, quote = "", None
    for ch in line:
        if quote:
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
        elif ch == "#":
            break
        out += ch
    return out.rstrip()


def load_yaml_subset(text):
    """Nested block mappings with `key: value` scalars / flow lists."""
    root = {}
    stack = [(-1, root)]
    for raw in text.splitlines():
        line = _strip_comment(raw)
        if not line.strip():
            continue
        indent = len(line) - len(line.lstrip(" "))
        key, sep, val = line.strip().partition(":")
        if not sep:
            raise ParamsError(f"cannot parse params line: {raw!r}")
        while stack and indent <= stack[-1][0]:
            stack.pop()
        parent = stack[-1][1]
        if val.strip() == "":
            child = {}
            parent[key.strip()] = child
            stack.append((indent, child))
        else:
            parent[key.strip()] = _flow(val)
    return root


def load_params(path):
    with open(path, "r") as f:
        text = f.read()
    try:
        import yaml  # noqa: F401
        return yaml.safe_load(text)
    except ImportError:
        return load_yaml_subset(text)


# ----------------------------------------------------------------------------- printing / timers
class Print:
    """Rank-0 console output (petgem/common.py:30-124); one process per GPU here."""

    @staticmethod
    def master(text, color_code=None):
        if int(os.environ.get("RANK", "0")) == 0:
            print(text)
            sys.stdout.flush()

    @staticmethod
    def header():
        Print.master("%" * 75)
        Print.master("%%%" + "PETGEM (GB300 forward-modelling hot path)".center(69) + "%%%")
        Print.master("%" * 75)


class Timer:
    def __init__(self, elapsed=0.0):
        self._start = 0.0
        self.elapsed = elapsed

    def start(self):
        self._start = time.time()

    def stop(self):
        if self._start > 0:
            self.elapsed += time.time() - self._start
            self._start = 0.0

    def reset(self):
        self.elapsed = 0.0


class _Timers:
    """Named wall-clock timers (petgem/common.py:367-473, same timer names)."""

    def __init__(self):
        self._elems = {}

    def __getitem__(self, key):
        return self._elems.setdefault(key, Timer())

    def __setitem__(self, key, value):
        self._elems[key] = Timer(value)

    def report(self):
        return {k: v.elapsed for k, v in self._elems.items()}


_TIMERS = _Timers()


def Timers(opath=None):
    """Process-wide timer registry (petgem's singleton ``Timers``)."""
    return _TIMERS


# ----------------------------------------------------------------------------- params
class InputParameters:
    """Params file loader and checker (petgem/common.py:129-361)."""

    def __init__(self, params, parEnv=None):
        inputs = load_params(params)
        try:
            self.model = inputs["model"]
            self.run = inputs["run"]
            self.output = inputs["output"]
        except (KeyError, TypeError):
            raise ParamsError("params file needs model, run and output sections")
        mode = self.model.get("mode")
        if mode is None:
            raise ParamsError("Modeling mode not provided. Please, verify the parameter file consistency.")
        if mode not in ("csem", "mt"):
            raise ParamsError("Modeling mode not supported.")
        if mode not in self.model:
            raise ParamsError(f"{mode} parameters not provided. Please, verify the parameter file consistency.")
        if mode == "csem":
            from_file, npol = self._verify_csem(self.model["csem"])
        else:
            from_file, npol = self._verify_mt(self.model["mt"])
        self.run["conductivity_from_file"] = from_file
        self.run["num_polarizations"] = npol
        for key in ("mesh", "receivers"):
            if key not in self.model:
                raise ParamsError(f"{key} parameter not provided. Please, verify the parameter file consistency.")
        if "nord" not in self.run:
            raise ParamsError("nord parameter not provided. Please, verify the parameter file consistency.")
        if not 1 <= int(self.run["nord"]) <= 6:
            raise ParamsError("Vector finite element basis order not supported. Please, select a valid order "
                              "(1,2,3,4,5,6).")
        if "cuda" not in self.run:
            self.run["cuda"] = False
        elif self.run["cuda"] not in (True, False):
            raise ParamsError("cuda option not supported. Please, select a valid order (True/False).")
        self.output.setdefault("vtk", False)
        if "directory" not in self.output:
            raise ParamsError("output directory parameter not provided. Please, verify the parameter file "
                              "consistency.")
        os.makedirs(self.output["directory"], exist_ok=True)
        if "directory_scratch" not in self.output:
            self.output["directory_scratch"] = self.output["directory"]
            self.output["remove_scratch"] = False
        else:
            os.makedirs(self.output["directory_scratch"], exist_ok=True)
            self.output["remove_scratch"] = True

    @staticmethod
    def _sigma_mode(i_sigma):
        if not isinstance(i_sigma, dict):
            raise ParamsError("sigma parameters invalid. Please, verify the parameter file consistency.")
        if "file" in i_sigma:
            if "horizontal" in i_sigma or "vertical" in i_sigma:
                raise ParamsError("sigma parameters invalid. Please, verify the parameter file consistency.")
            return True
        if "horizontal" in i_sigma and "vertical" in i_sigma:
            return False
        raise ParamsError("sigma parameters invalid. Please, verify the parameter file consistency.")

    def _verify_csem(self, csem):
        if "sigma" not in csem:
            raise ParamsError("csem parameters not provided. Please, verify the parameter file consistency.")
        from_file = self._sigma_mode(csem["sigma"])
        if "source" not in csem:
            raise ParamsError("source parameters not provided. Please, verify the parameter file consistency.")
        src = csem["source"]
        if len(src) != 6:
            raise ParamsError("number of source parameters is not consistent. Please, verify the parameter file "
                              "consistency.")
        for k in ("frequency", "position", "azimuth", "dip", "current", "length"):
            if k not in src:
                raise ParamsError(f"{k} parameter not provided. Please, verify the parameter file consistency.")
        return from_file, 1

    def _verify_mt(self, mt):
        if "sigma" not in mt:
            raise ParamsError("mt parameters not provided. Please, verify the parameter file consistency.")
        from_file = self._sigma_mode(mt["sigma"])
        for k in ("frequency", "polarization"):
            if k not in mt:
                raise ParamsError(f"{k} parameter not provided for model. Please, verify the parameter file "
                                  "consistency.")
        return from_file, len(mt["polarization"])


def parse_petsc_options(argv_or_path):
    """KSP options of the subset petgem's options files use (-ksp_type,
    -ksp_rtol, -ksp_max_it, -ksp_gmres_restart, -pc_type) plus this library's
    -pg_precision {fp64,mixed,df64} and -pg_nrhs.  Accepts an options file path or
    an argv list containing -options_file."""
    tokens = []
    if isinstance(argv_or_path, str):
        paths = [argv_or_path]
        argv = []
    else:
        argv = list(argv_or_path)
        paths = [argv[i + 1] for i, a in enumerate(argv[:-1]) if a == "-options_file"]
    for pth in paths:
        with open(pth) as f:
            for ln in f:
                ln = ln.split("#")[0].strip()
                if ln:
                    tokens += ln.split()
    i = 0
    while i < len(argv):
        if argv[i] == "-options_file":
            i += 2
            continue
        if argv[i].startswith("-"):
            tokens.append(argv[i])
            if i + 1 < len(argv) and not argv[i + 1].startswith("-") and not argv[i + 1].endswith((".yaml", ".yml")):
                tokens.append(argv[i + 1])
                i += 1
        i += 1
    opts = {}
    i = 0
    while i < len(tokens):
        t = tokens[i]
        if t.startswith("-"):
            val = tokens[i + 1] if i + 1 < len(tokens) and not tokens[i + 1].startswith("-") else True
            opts[t[1:]] = val
            i += 2 if val is not True else 1
        else:
            i += 1
    return opts


__all__ = ["InputParameters", "ParamsError", "Print", "Timers", "Timer", "load_params", "parse_petsc_options"]
