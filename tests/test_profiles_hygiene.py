"""The profile summaries under profiles/ are short text, and every ncu command they give leaves
the GPU clocks alone (--clock-control none) and runs committed files only."""
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
