"""The integration example stays true, as the reference keeps its guide's code identical to code that builds
(IntegrationGuideTests.swift:90-124): the world-API example below (the one a port of the guide shows) runs as written
against a stand-in device world that forwards to the oracle, and every `bp_*` entry point the serving example calls is
declared in the public header."""
import re
from pathlib import Path

from bubblephysics_gb300 import world as W
from test_world_api_oracle_cpu import OracleBackedWorld

ROOT = Path(__file__).resolve().parent.parent

PYTHON_EXAMPLE = """
from bubblephysics_gb300.world import *
world = BubbleWorld(WorldConfiguration(simulation_region=(0, 0, 375, 700)))
world.submit(WorldTransaction()
             .update_physics_material("soft", PhysicsMaterial(contact_stiffness=229.0))
             .add(RigidBodyDescriptor(100, Circle(30.0), (180.0, 300.0)))
             .add(BubbleDescriptor(1, (100.0, 100.0), 12.0, 8.0, "soft", velocity=(30.0, 0.0),
                                   event_interest=frozenset({EventInterest.CONTACT}))))
frame = world.advance(1 / 60)          # one fixed step; frame.objects[1].position, frame.events
"""

C_SERVING_EXAMPLE = """
bp_server_config cfg = {0};
cfg.max_worlds = world_count;
bp_server* server;
bp_server_create(context, &cfg, &server);
for (uint32_t w = 0; w < world_count; ++w) bp_server_add_world(server, &descs[w], &inputs[w], NULL);
bp_server_submit(server, world, 1, &request_id);
uint32_t finished;
bp_server_progress(server, 200, &finished);
bp_server_completion done[256];
uint32_t n;
bp_server_poll(server, done, 256, &n);
bp_server_read_bubbles(server, world, bubbles, capacity, &count);
"""


def test_the_python_example_runs_as_written(monkeypatch):
    monkeypatch.setattr(W, "World", OracleBackedWorld)
    monkeypatch.setattr(W, "default_context", lambda: None)
    scope = {}
    exec(compile(PYTHON_EXAMPLE, "world_api_example", "exec"), scope)
    frame, world = scope["frame"], scope["world"]
    assert frame.step_index == 1 and world.diagnostics.last_advance_issue is None
    assert len(frame.transaction_receipts) == 1 and set(frame.objects) == {1, 100}


def test_every_entry_point_the_c_example_names_is_declared():
    header = (ROOT / "include" / "bubblephysics.h").read_text()
    declared = set(re.findall(r"\b(bp_[a-z0-9_]+)\s*\(", header))
    named = set(re.findall(r"\b(bp_[a-z0-9_]+)\s*\(", C_SERVING_EXAMPLE))
    assert named and named <= declared, named - declared
