"""The committed ncu summaries (profiles/) each give the command that made
them; the scripts those commands run are files of this repository, and every
ncu invocation leaves the GPU clocks alone (--clock-control none)."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def profile_texts():
    paths = sorted(glob.glob(os.path.join(ROOT, "profiles", "*")))
    assert paths
    for p in paths:
        with open(p) as f:
            yield os.path.basename(p), f.read()


def test_profiles_cite_committed_scripts_and_keep_clocks():
    for name, text in profile_texts():
        assert "ncu" in text, name  # the command that made it
        for script in re.findall(r"python3?\s+([\w./-]+\.py)", text):
            assert os.path.exists(os.path.join(ROOT, script)), (name, script)
            assert not script.startswith("_work"), (name, script)
        for cmd in re.findall(r"\bncu\b[^\n]*(?:\\\n[^\n]*)*", text):
            if "--metrics" in cmd or "--set" in cmd or "--section" in cmd:
                assert "--clock-control none" in cmd, (name, cmd)
