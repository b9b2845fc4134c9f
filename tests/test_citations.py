"""Every `<file>.jl:N` citation in the repository points at a line that
exists in the reference, and the constructor / kernel anchors the host and
the oracle cite sit where they are cited.

Reads the reference sources from SC_REFERENCE_ROOT (default: the read-only
mount of SpaceCharge.jl in the build container, /root/reference); skipped
where the reference is absent.
"""
from __future__ import annotations

import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("SC_REFERENCE_ROOT", "/root/reference")

# files whose citations are this repository's own statements (the build's
# planning notes are written by others and quote the reference themselves)
SKIP_FILES = {"SURVEY.md", "VERDICT.md", "ADVICE.md", "BASELINE.md", "BASELINE.json"}
SKIP_DIRS = {".git", "_work", "gpurun_out", "_build", "lib", "__pycache__", "baseline", ".pytest_cache"}
CITE = re.compile(r"((?:[\w.]+/)*)(\w+\.jl):(\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*)")

# (file, line, text the line starts with after stripping indentation)
ANCHORS = [
    ("src/mesh.jl", 19, "mutable struct Mesh3D"),
    ("src/mesh.jl", 49, "function _get_workspace"),
    ("src/mesh.jl", 95, "function Mesh3D("),
    ("src/mesh.jl", 100, "T::Type{<:AbstractFloat}=Float64"),
    ("src/mesh.jl", 107, 'error("All elements of grid_size must be at least 2.")'),
    ("src/mesh.jl", 111, 'error("Particle arrays cannot be empty.")'),
    ("src/mesh.jl", 115, 'error("Particle coordinate arrays must have the same length.")'),
    ("src/mesh.jl", 120, "x_min, x_max = extrema(particles_x)"),
    ("src/mesh.jl", 196, "function Mesh3D("),
    ("src/mesh.jl", 210, 'error("max_bounds must be strictly greater than min_bounds for all dimensions.")'),
    ("src/mesh.jl", 220, "delta = (cv_max_bounds .- cv_min_bounds) ./ (grid_size .- 1)"),
    ("src/mesh.jl", 240, "function Base.show"),
    ("src/deposition.jl", 10, "function clear_mesh!"),
    ("src/deposition.jl", 28, "function deposit_particle!("),
    ("src/deposition.jl", 218, "function deposit!("),
    ("src/green_functions.jl", 13, "@inline function potential_green_function"),
    ("src/green_functions.jl", 35, "@inline function field_green_function"),
    ("src/green_functions.jl", 69, "@kernel function get_green_kernel!"),
    ("src/green_functions.jl", 103, "@kernel function apply_8point_differencing!"),
    ("src/solvers/free_space.jl", 14, "function solve!("),
    ("src/solvers/free_space.jl", 56, "function solve_freespace!("),
]


def _ref_index():
    idx = {}
    for d, dirs, fs in os.walk(REF):
        dirs[:] = [x for x in dirs if x != ".git"]
        for f in fs:
            if f.endswith(".jl"):
                idx.setdefault(f, []).append(os.path.join(d, f))
    return idx


def _repo_texts():
    for d, dirs, fs in os.walk(ROOT):
        dirs[:] = [x for x in dirs if x not in SKIP_DIRS]
        for f in fs:
            if f in SKIP_FILES or f.endswith((".so", ".o", ".pyc", ".json", ".csv")):
                continue
            p = os.path.join(d, f)
            try:
                with open(p, encoding="utf-8") as fh:
                    yield p, fh.read()
            except (UnicodeDecodeError, OSError):
                continue


needs_ref = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference sources not present")


@needs_ref
def test_every_citation_is_in_range():
    idx = _ref_index()
    lengths = {}
    bad, total = [], 0
    for path, text in _repo_texts():
        for ln, line in enumerate(text.splitlines(), 1):
            for m in CITE.finditer(line):
                base = m.group(2)
                if base not in idx:
                    continue  # a file of this repository (the Julia wrapper), not the reference's
                cands = [c for c in idx[base] if c.endswith(m.group(1) + base)] or idx[base]
                ref = cands[0]
                if ref not in lengths:
                    with open(ref, encoding="utf-8") as fh:
                        lengths[ref] = sum(1 for _ in fh)
                for part in re.split(r",\s?", m.group(3)):
                    nums = [int(x) for x in part.split("-")]
                    total += 1
                    if max(nums) > lengths[ref] or min(nums) < 1 or (len(nums) == 2 and nums[0] > nums[1]):
                        bad.append(f"{os.path.relpath(path, ROOT)}:{ln}: {m.group(0)} ({lengths[ref]} lines)")
    assert total > 100, f"only {total} citations found"
    assert not bad, "citations past the end of the cited file:\n" + "\n".join(bad)


@needs_ref
@pytest.mark.parametrize("rel,line,start", ANCHORS)
def test_anchor_lines(rel, line, start):
    with open(os.path.join(REF, rel), encoding="utf-8") as fh:
        lines = fh.read().splitlines()
    assert lines[line - 1].strip().startswith(start), f"{rel}:{line} is {lines[line - 1].strip()!r}"
