"""Spectra (``.ev``) and vertex-function (PSOL) text files, as written and
read by ``lapy.io`` (lapy/io.py:10-310), so that descriptors computed here
can be exchanged with the reference and with ShapeDNA tools.

Host code: these are small text files around the GPU path.  The formats are
reproduced exactly, including the reference's quirks: the writer labels the
timing lines ``Time(Pre) :`` / ``Time(calcAB) :`` / ``Time(calcEW) :`` (with
a space before the colon), which its own reader does not pick up again.
"""

from __future__ import annotations

import logging
import re

import numpy as np

logger = logging.getLogger(__name__)

# header fields of an .ev file and their types (lapy/io.py:96-124)
_EV_INT = ("Creator", "File", "User", "Refine", "Degree", "Dimension", "Elements", "DoF", "NumEW",
           "EulerChar", "Time(pre)", "Time(calcAB)", "Time(calcEW)")
_EV_FLOAT = ("Area", "Volume", "BLength")
_EV_LABEL = {"Time(pre)": "TimePre", "Time(calcAB)": "TimeCalcAB", "Time(calcEW)": "TimeCalcEW"}


def read_vfunc(filename: str) -> list[float]:
    """Vertex function from a PSOL text file (lapy/io.py:10-52): a line
    ``Solution:`` and values separated by ``,`` or ``;``, optionally in
    ``()`` or ``{}`` brackets, on one line or one per line."""
    try:
        with open(filename) as fh:
            lines = [ln.strip() for ln in fh]
    except OSError:
        logger.error("File %s not found or not readable", filename)
        raise
    if "Solution:" not in lines:
        raise ValueError(f"Expected 'Solution:' marker in {filename}")
    lines.remove("Solution:")
    body = [re.sub(r"[{()}]", "", ln) for ln in lines if ln]
    if not body:
        raise ValueError(f"No vertex function data found in {filename}")
    if len(body) == 1:
        body = re.split(r"[,;]", body[0])
    return [float(x) for x in body]


def write_vfunc(filename: str, vfunc: np.ndarray) -> None:
    """PSOL file: ``Solution:`` then the values, comma separated in ``()``
    (lapy/io.py:286-310)."""
    try:
        fh = open(filename, "w")
    except OSError:
        logger.error("File %s not writable", filename)
        raise
    with fh:
        fh.write("Solution:\n")
        fh.write("(" + ",".join(np.asarray(vfunc).astype(str)) + ")")


def _braced(lines: list[str], i: int, strip_parens: bool) -> tuple[str, int]:
    """Text between the next ``{`` and the matching ``}`` (joined over lines,
    braces removed) and the index of the closing line."""
    while lines[i].find("{") < 0:
        i += 1
    parts = []
    while True:
        seg = lines[i].strip().replace("{", "").replace("}", "")
        if strip_parens:
            seg = seg.replace("(", "").replace(")", "")
        parts.append(seg)
        if lines[i].find("}") >= 0:
            return "".join(parts), i
        i += 1


def read_ev(filename: str) -> dict:
    """Header fields, ``Eigenvalues`` and (when present) ``Eigenvectors``
    (n x k) and ``EigenvectorsSize`` of an .ev file (lapy/io.py:55-182)."""
    try:
        with open(filename) as fh:
            lines = fh.read().splitlines()
    except OSError:
        logger.error("File %s not readable", filename)
        raise
    d: dict = {}
    i = 0
    while i < len(lines):
        line = lines[i].lstrip()
        if ":" in line:
            key = line.split(":", 1)[0]
            if key in _EV_INT or key in _EV_FLOAT:
                cast = float if key in _EV_FLOAT else int
                d[_EV_LABEL.get(key, key)] = cast(lines[i].split(":", 1)[1].strip())
                i += 1
                continue
        if line.startswith("Eigenvalues"):
            text, i = _braced(lines, i + 1, strip_parens=False)
            d["Eigenvalues"] = np.array(text.split(";")).astype(float)
            i += 1
        elif line.startswith("Eigenvectors"):
            i += 1
            while not lines[i].strip().startswith("sizes"):
                i += 1
            sizes = np.array(lines[i].strip().split()[1:]).astype(int)
            d["EigenvectorsSize"] = sizes
            text, i = _braced(lines, i + 1, strip_parens=True)
            vals = np.array(text.replace(";", " ").replace(",", " ").split()).astype(float)
            if len(vals) == sizes[0] * sizes[1]:
                # stored one eigenvector (column) after another
                d["Eigenvectors"] = vals.reshape(sizes[1], sizes[0]).T
            else:
                logger.warning("Length of eigenvectors is not %d times %d.", sizes[0], sizes[1])
            i += 1
        else:
            i += 1
    return d


def write_ev(filename: str, d: dict) -> None:
    """.ev file in ShapeDNA's text format (lapy/io.py:185-283): header fields
    that are present, the eigenvalues, and the eigenvectors one column per
    parenthesised group."""
    try:
        fh = open(filename, "w")
    except OSError:
        logger.error("File %s not writable", filename)
        raise
    with fh:
        if "Eigenvalues" not in d:
            raise ValueError("ERROR: no Eigenvalues specified")
        out = []
        for key in ("Creator", "File", "User"):
            if key in d:
                out.append(f" {key}: {d[key]}\n")
        for key in ("Refine", "Degree", "Dimension", "Elements", "DoF", "NumEW"):
            if key in d:
                out.append(f" {key}: {d[key]!s}\n")
        out.append("\n")
        for key in ("Area", "Volume", "BLength", "EulerChar"):
            if key in d:
                out.append(f" {key}: {d[key]!s}\n")
        out.append("\n")
        for key, label in (("TimePre", "Time(Pre)"), ("TimeCalcAB", "Time(calcAB)"), ("TimeCalcEW", "Time(calcEW)")):
            if key in d:
                out.append(f" {label} : {d[key]!s}\n")
        if all(k in d for k in ("TimePre", "TimeCalcAB", "TimeCalcEW")):
            out.append(f" Time(total ) : {d['TimePre'] + d['TimeCalcAB'] + d['TimeCalcEW']!s}\n")
        out.append("\n")
        out.append("Eigenvalues:\n")
        out.append("{ " + " ; ".join(str(x) for x in d["Eigenvalues"]) + " }\n")
        out.append("\n")
        if "Eigenvectors" in d:
            ev = d["Eigenvectors"]
            out.append("Eigenvectors:\n")
            out.append("sizes: " + " ".join(str(s) for s in ev.shape) + "\n")
            out.append("\n")
            cols = ["(" + ",".join(str(x) for x in ev[:, j]) + ")" for j in range(ev.shape[1])]
            out.append("{ " + " ;\n".join(cols) + " }\n")
        fh.write("".join(out))
