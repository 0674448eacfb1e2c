"""The committed ncu summaries (profiles/) each give the command that made
them; the scripts those commands run are files of this repository, every
ncu invocation leaves the GPU clocks alone (--clock-control none), and every
capture that collects more than the launch list's gpu__time_duration.sum
names a single kernel (-k) and at most four launches (-c)."""
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


def _collects_more_than_durations(cmd):
    if "--set" in cmd or "--section" in cmd:
        return True
    m = re.search(r"--metrics\s+(\S+)", cmd)
    return bool(m) and set(m.group(1).split(",")) != {"gpu__time_duration.sum"}


def test_metric_captures_are_one_kernel_few_launches():
    for name, text in profile_texts():
        for cmd in re.findall(r"\bncu\b[^\n]*(?:\\\n[^\n]*)*", text):
            if not _collects_more_than_durations(cmd):
                continue
            k = re.search(r"-k\s+(?:regex:)?\"?([^\s\"]+)\"?", cmd)
            assert k and "|" not in k.group(1), (name, cmd)
            c = re.search(r"-c\s+(\d+)", cmd)
            assert c and int(c.group(1)) <= 4, (name, cmd)
