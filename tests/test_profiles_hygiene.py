"""The profile summaries under profiles/ are short text, and every ncu command they give leaves
the GPU clocks alone (--clock-control none) and runs committed files only; no source file
reaches into the scratch folder or names the batched copy calls."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROFILES = os.path.join(ROOT, "profiles")


def profile_files():
    return sorted(os.path.join(PROFILES, f) for f in os.listdir(PROFILES))


def test_profiles_are_short_text_summaries():
    for path in profile_files():
        assert os.path.splitext(path)[1] in (".md", ".txt", ".json"), path
        assert os.path.getsize(path) < 64 * 1024, path


def test_every_ncu_command_keeps_the_clocks_and_runs_committed_files():
    commands = []
    for path in profile_files():
        text = open(path).read()
        commands += [(path, m.group(0)) for m in re.finditer(r"\bncu (?:--|-[a-zA-Z])[^`\"\n]*", text)]
    assert commands
    for path, cmd in commands:
        assert "--clock-control none" in cmd, (path, cmd)
        assert "_work/" not in cmd and "/root/" not in cmd, (path, cmd)


def tracked_sources():
    import subprocess
    try:
        out = subprocess.run(["git", "-C", ROOT, "ls-files"], capture_output=True, text=True, check=True).stdout
    except (OSError, subprocess.CalledProcessError):
        return None
    keep = (".py", ".cu", ".cuh", ".cpp", ".h", ".inc", ".c", "Makefile")
    return [os.path.join(ROOT, f) for f in out.splitlines() if f.endswith(keep)]


def test_sources_do_not_reach_into_scratch_or_name_closed_calls():
    import pytest
    files = tracked_sources()
    if not files:
        pytest.skip("not a git checkout")
    # the batched host-device copy entry points are not used anywhere: no source may name them
    closed = re.compile("cu(?:da)?Memcpy(?:3D)?Batch" + "Async")
    this = os.path.abspath(__file__)
    for path in files:
        if os.path.abspath(path) == this or not os.path.exists(path):
            continue
        text = open(path, errors="replace").read()
        assert "_work/" not in text, path
        assert not closed.search(text), path
