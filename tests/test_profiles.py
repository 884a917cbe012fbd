"""The DRAM traffic figures bench.py reports beside its roofline come from ncu
summaries committed under profiles/: every cited summary exists, and it
quotes the same bytes (its DRAM read and write lines, or their total to
0.1 MB)."""
import re
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def _quoted(text: str, nbytes: int) -> bool:
    rd = re.search(r"DRAM read \| ([0-9.]+) Mbyte", text)
    wr = re.search(r"DRAM write \| ([0-9.]+) Mbyte", text)
    if rd and wr and abs((float(rd.group(1)) + float(wr.group(1))) * 1e6 - nbytes) < 2:
        return True
    return f"{nbytes / 1e6:.1f} MB" in text


def test_cited_traffic_is_in_the_profiles():
    cited = list(bench.SPMV_TRAFFIC.values()) + list(bench.SSOR_TRAFFIC.values())
    assert cited
    for nbytes, path in cited:
        f = ROOT / path
        assert f.is_file(), path
        assert _quoted(f.read_text(), nbytes), (path, nbytes)
