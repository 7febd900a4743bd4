"""The integration notes' examples stay true, as the reference keeps its guide's code identical to code that builds
(IntegrationGuideTests.swift:90-124): the Python block of INTEGRATION.md runs as written against a stand-in device
world that forwards to the oracle, and every `bp_*` entry point the C block names is declared in the public header."""
import re
from pathlib import Path

import pytest

from bubblephysics_gb300 import world as W
from test_world_api_oracle_cpu import OracleBackedWorld

ROOT = Path(__file__).resolve().parent.parent


def blocks(language):
    text = (ROOT / "INTEGRATION.md").read_text()
    return re.findall(r"```" + language + r"\n(.*?)```", text, re.S)


def test_the_python_example_runs_as_written(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)
    (code,) = blocks("python")
    scope = {}
    exec(compile(code, "INTEGRATION.md", "exec"), scope)
    frame, world = scope["frame"], scope["world"]
    assert frame.step_index == 1 and world.diagnostics.last_advance_issue is None
    assert len(frame.transaction_receipts) == 1 and set(frame.objects) == {1, 100}


def test_every_entry_point_the_c_example_names_is_declared():
    header = (ROOT / "include" / "bubblephysics.h").read_text()
    declared = set(re.findall(r"\b(bp_[a-z0-9_]+)\s*\(", header))
    named = {name for code in blocks("c") for name in re.findall(r"\b(bp_[a-z0-9_]+)\s*\(", code)}
    assert named and named <= declared, named - declared
