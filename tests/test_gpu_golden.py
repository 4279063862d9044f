"""Full-size parity of the CUDA path against the committed golden digests of
the oracle (tests/golden/golden.json): for config 1 (1,000 circles), config
2a (65,535 layers, 2560x1600), config 2 (100,000 layers, widened format)
and config 3 (50,000 glyph layers, 3840x2160), the canonical pixel segments
(count, NONE slots, SHA-256) and the RGBA8 frame (SHA-256) are bit-exact."""
import pytest

from tests.golden import make_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", list(make_golden.CASES))
def test_gpu_matches_golden(gpu_lib, name):
    import torch
    from cassia_gb300 import Composition, scenes
    want = make_golden.load()["cases"][name]
    sc = make_golden.make_scene(name)
    c = Composition(wide=sc.wide)
    scenes.load(sc, c)
    segs, none = c.pixel_segments(canonical=True)
    assert (len(segs), none) == (want["segments"], want["none"])
    assert make_golden.digest(segs.astype("<u8")) == want["segments_sha256"]
    del segs
    out = torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8, device="cuda")
    c.render(out.data_ptr(), sc.width, sc.background, height=sc.height)
    assert make_golden.digest(out.cpu().numpy()) == want["rgba_sha256"]
    # and replayed from a frame graph
    c.set_graph_mode(True)
    for _ in range(2):
        out.zero_()
        c.render(out.data_ptr(), sc.width, sc.background, height=sc.height)
    assert c.stats()["graph_replayed"] == 1
    assert make_golden.digest(out.cpu().numpy()) == want["rgba_sha256"]
    c.close()
