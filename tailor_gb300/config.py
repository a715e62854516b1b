"""Case configuration: the reference's config.yaml, parsed and validated.

``load_config(path)`` returns a :class:`Config` with the reference
``Recipe`` fields (src/CPlusPlus/Recipe.hpp:17-61), parsed and checked as
``Parser::parseOnRoot`` does (src/CPlusPlus/Parser.cpp:37-148): required
keys, the FD-q cache path derived from the source file
(``<source dir>/FD-q/fdq_<stem>_qy<q_y>_qz<q_z>.h5``), finite values and
the physical ranges, with the reference's messages.

No YAML library is installed here, so the file is read by a small parser
for the subset such configuration files use: block mappings by
indentation, ``key: value`` scalars (integers, floats, plain or quoted
strings), comments and blank lines.  Anything outside that subset (flow
collections, sequences, anchors, multi-line scalars) is rejected with a
line number rather than misread.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass
from pathlib import Path

from .case import Physics


class ConfigError(ValueError):
    pass


def _scalar(text: str, lineno: int):
    t = text.strip()
    if not t:
        return None
    if t[0] in "'\"":
        q = t[0]
        if len(t) < 2 or t[-1] != q:
            raise ConfigError(f"line {lineno}: unterminated quoted scalar")
        body = t[1:-1]
        return body.replace("''", "'") if q == "'" else bytes(body, "utf-8").decode(
            "unicode_escape")
    if t[0] in "[{&*!|>" or t.startswith("- "):
        raise ConfigError(f"line {lineno}: unsupported YAML construct {t[:12]!r}")
    if re.fullmatch(r"[-+]?\d+", t):
        return int(t)
    if re.fullmatch(r"[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?", t):
        return float(t)
    low = t.lower()
    if low in (".inf", "+.inf"):
        return math.inf
    if low == "-.inf":
        return -math.inf
    if low == ".nan":
        return math.nan
    if low in ("true", "false"):
        return low == "true"
    if low in ("null", "~"):
        return None
    return t


def _strip_comment(line: str) -> str:
    """The line without its comment: a '#' at the start of the line or after
    whitespace, outside quotes.  A quote opens a quoted scalar only where a
    key or a value begins, so apostrophes inside plain scalars are text."""
    out, quote, i, n = [], None, 0, len(line)
    at_start = True  # the next non-blank character begins a key or a value
    while i < n:
        ch = line[i]
        if quote:
            out.append(ch)
            if quote == "'" and ch == "'" and line[i + 1:i + 2] == "'":
                out.append("'")  # '' inside a single-quoted scalar
                i += 2
                continue
            if quote == '"' and ch == "\\" and i + 1 < n:
                out.append(line[i + 1])
                i += 2
                continue
            if ch == quote:
                quote = None
            i += 1
            continue
        if ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        if ch in "'\"" and at_start:
            quote = ch
        if ch == ":" and line[i + 1:i + 2] in ("", " ", "\t"):
            at_start = True
        elif ch not in " \t":
            at_start = False
        out.append(ch)
        i += 1
    return "".join(out).rstrip()


def parse_yaml(text: str) -> dict:
    """Block-mapping YAML subset -> nested dicts."""
    root: dict = {}
    stack: list[tuple[int, dict]] = [(0, root)]  # (indent of the mapping's keys, mapping)
    pending: tuple[str, dict] | None = None      # key whose value may be a nested mapping
    for lineno, raw in enumerate(text.splitlines(), 1):
        lead = raw[:len(raw) - len(raw.lstrip())]
        if "\t" in lead:
            raise ConfigError(f"line {lineno}: tabs are not allowed in indentation")
        line = _strip_comment(raw)
        if not line.strip() or line.strip() in ("---", "..."):
            continue
        indent = len(line) - len(line.lstrip(" "))
        m = re.fullmatch(r"((?:\"[^\"]*\")|(?:'[^']*')|[^:#'\"\s][^:]*?)\s*:(?:\s+(.*))?",
                         line.strip())
        if not m:
            raise ConfigError(f"line {lineno}: expected 'key: value'")
        key = m.group(1).strip().strip("'\"")
        if pending is not None:
            pkey, pmap = pending
            if indent > stack[-1][0]:
                child: dict = {}
                pmap[pkey] = child
                stack.append((indent, child))
            pending = None
        while indent < stack[-1][0]:
            stack.pop()
        if indent != stack[-1][0]:
            raise ConfigError(f"line {lineno}: bad indentation")
        cur = stack[-1][1]
        if key in cur:
            raise ConfigError(f"line {lineno}: duplicate key {key!r}")
        value = m.group(2)
        if value is None or not value.strip():
            cur[key] = None
            pending = (key, cur)
        else:
            cur[key] = _scalar(value, lineno)
    return root


@dataclass
class Config:
    case_title: str
    q_y: int
    q_z: int
    source_file: Path
    input_file: Path
    output_file: Path
    physics: Physics


def _req(node, key: str, kind):
    if not isinstance(node, dict) or key not in node or node[key] is None:
        raise ConfigError(f"Missing YAML key: {key}")
    v = node[key]
    if kind is int:
        if isinstance(v, bool) or not isinstance(v, int):
            raise ConfigError(f"YAML key {key} must be an integer")
        return v
    if kind is float:
        if isinstance(v, bool) or not isinstance(v, (int, float)):
            raise ConfigError(f"YAML key {key} must be a number")
        return float(v)
    return str(v)


def _mapping(root: dict, key: str, label: str | None = None) -> dict:
    v = root.get(key) if isinstance(root, dict) else None
    if not isinstance(v, dict):
        raise ConfigError(f"Missing or invalid YAML mapping: {label or key}")
    return v


def load_config(path: str | Path, require_input: bool = False) -> Config:
    """Parse and validate a case configuration (Parser.cpp:37-148).
    With require_input the prepared FD-q file must exist, as the reference's
    C++ solver requires; the launcher prepares it otherwise."""
    cfg_path = Path(path).absolute()
    root = parse_yaml(cfg_path.read_text())
    title = _req(root, "CaseTitle", str)
    q = _mapping(root, "Q-Value")
    q_y, q_z = _req(q, "y", int), _req(q, "z", int)
    folder, file = Path(_req(root, "Folder", str)), Path(_req(root, "File", str))
    source = file if file.is_absolute() else cfg_path.parent / folder / file
    source = Path(_normalize(source))
    input_file = source.parent / "FD-q" / f"fdq_{source.stem}_qy{q_y}_qz{q_z}.h5"
    stab = root.get("Stability")
    alpha = stab.get("Alpha") if isinstance(stab, dict) else None
    if not isinstance(alpha, dict):
        raise ConfigError("Missing YAML key: Stability.Alpha")
    a = complex(_req(alpha, "Real", float), _req(alpha, "Imag", float))
    es = _mapping(root, "EigenSolver")
    sc = _mapping(es, "SearchCenterOmega", "EigenSolver.SearchCenterOmega")
    omega = complex(_req(sc, "Real", float), _req(sc, "Imag", float))
    nev = _req(es, "NumberOfEigenvalues", int)
    tol = _req(es, "Tolerance", float)
    max_it = _req(es, "MaximumIterations", int)
    out = _mapping(root, "Output")
    out_file = Path(_req(out, "File", str))
    out_file = Path(_normalize(out_file if out_file.is_absolute() else cfg_path.parent / out_file))
    phys = root.get("Physics") if isinstance(root.get("Physics"), dict) else {}
    tg = phys.get("Targets") if isinstance(phys.get("Targets"), dict) else {}
    gas = phys.get("Gas") if isinstance(phys.get("Gas"), dict) else {}
    tr = phys.get("Transport") if isinstance(phys.get("Transport"), dict) else {}
    ph = Physics(reynolds=_req(tg, "ReynoldsNumber", float), mach=_req(tg, "MachNumber", float),
                 prandtl=_req(gas, "PrandtlNumber", float),
                 gas_constant=_req(gas, "GasConstant", float),
                 gamma=_req(gas, "RatioOfSpecificHeats", float),
                 reference_viscosity=_req(tr, "ReferenceMu", float),
                 reference_temperature=_req(tr, "ReferenceTemperature", float),
                 sutherland_constant=_req(tr, "SutherlandConstant", float),
                 alpha=a, omega=omega, nev=nev, tol=tol, max_it=max_it)
    if q_y < 2 or q_z < 2:
        raise ConfigError("Q-Value.y and Q-Value.z must both be at least 2")
    if require_input and not input_file.is_file():
        raise ConfigError(f"FD-q input file does not exist: {input_file}. "
                          f"Run Tailor.py -c {cfg_path} first")
    for v, name in ((a.real, "Stability.Alpha.Real"), (a.imag, "Stability.Alpha.Imag"),
                    (omega.real, "EigenSolver.SearchCenterOmega.Real"),
                    (omega.imag, "EigenSolver.SearchCenterOmega.Imag"),
                    (tol, "EigenSolver.Tolerance"), (ph.reynolds, "ReynoldsNumber"),
                    (ph.mach, "MachNumber"), (ph.prandtl, "PrandtlNumber"),
                    (ph.gas_constant, "GasConstant"), (ph.gamma, "RatioOfSpecificHeats"),
                    (ph.reference_viscosity, "ReferenceMu"),
                    (ph.reference_temperature, "ReferenceTemperature"),
                    (ph.sutherland_constant, "SutherlandConstant")):
        if not math.isfinite(v):
            raise ConfigError(f"{name} must be finite")
    if (ph.reynolds <= 0 or ph.mach <= 0 or ph.prandtl <= 0 or ph.gas_constant <= 0
            or ph.gamma <= 1 or ph.reference_viscosity <= 0 or ph.reference_temperature <= 0
            or ph.sutherland_constant < 0):
        raise ConfigError("The physical parameters in config.yaml are outside their valid ranges")
    if nev <= 0 or tol <= 0 or max_it <= 0:
        raise ConfigError("EigenSolver counts, tolerance, and iteration limit must be positive")
    return Config(title, q_y, q_z, source, input_file, out_file, ph)


def _normalize(p: Path) -> str:
    import os
    return os.path.normpath(str(p))
