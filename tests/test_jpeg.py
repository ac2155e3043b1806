"""JPEG decoding of the glTF ingest (rt_jpeg_decode), on streams written by tests/jpeg_writer.py.

The reference decodes every image format gltf::import supports (rustracer-core/src/loader.rs:36-113,
266); JPEG comes from the `image` crate.  Checks: the decoded image is the encoded one within the
quantisation error; progressive files (spectral selection, and successive approximation of DC and AC
coefficients) decode to exactly the baseline file's image, since they carry the same quantised
coefficients; restart intervals, 4:2:0 chroma and grey frames; ragged sizes; refusal of streams the
decoder does not handle; and two real-world photographs.
"""
from pathlib import Path

import numpy as np
import pytest

from jpeg_writer import encode_baseline, encode_progressive
from rustracer_gb300 import _abi as A
from rustracer_gb300 import gltf


def decode(data: bytes) -> np.ndarray:
    t = gltf.decode_jpeg(data)
    assert t is not None, A.load().rt_last_error()
    return np.rint(np.asarray(t.data) * 255.0).astype(np.int64).reshape(t.height, t.width, 4)


def image(h, w, seed=0, smooth_chroma=False):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    base = 128 + 80 * np.sin(x / 7.0) * np.cos(y / 5.0)
    if smooth_chroma:  # detail in luma only; the colour drifts slowly (what 4:2:0 keeps)
        img = np.stack([base + 25 * np.cos(x / 40.0), base, base + 25 * np.sin(y / 30.0)], -1)
    else:
        img = np.stack([base + 30 * np.cos(x / 11.0), base * 0.8 + 40 * np.sin(y / 9.0), 255 - base * 0.7], -1)
        img += rng.normal(0, 6, img.shape)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


Q_FINE = np.ones(64, np.int64)
Q_COARSE = (np.add.outer(np.arange(8), np.arange(8)).reshape(64) * 3 + 4).astype(np.int64)


@pytest.mark.parametrize("h,w", [(16, 16), (29, 37), (61, 90)])
def test_baseline_444_roundtrip(lib, h, w):
    img = image(h, w)
    out = decode(encode_baseline(img, Q_FINE))
    assert out.shape == (h, w, 4) and (out[..., 3] == 255).all()
    err = np.abs(out[..., :3] - img.astype(np.int64))
    assert err.max() <= 4 and err.mean() < 1.0, (err.max(), err.mean())


def test_baseline_420_and_restart(lib):
    img = image(45, 70, smooth_chroma=True)
    plain = decode(encode_baseline(img, Q_FINE, subsample=True))
    err = np.abs(plain[..., :3] - img.astype(np.int64))
    assert err.mean() < 1.5 and err.max() <= 8, (err.mean(), err.max())
    # restart markers every 3 MCUs: the same image
    assert np.array_equal(decode(encode_baseline(img, Q_FINE, subsample=True, restart=3)), plain)


def test_grey(lib):
    img = image(33, 41)[..., 1]
    out = decode(encode_baseline(img, Q_FINE))
    assert (out[..., 0] == out[..., 1]).all() and (out[..., 1] == out[..., 2]).all()
    assert np.abs(out[..., 0] - img.astype(np.int64)).max() <= 2


@pytest.mark.parametrize("subsample", [False, True])
@pytest.mark.parametrize("approx", [False, True])
def test_progressive_equals_baseline(lib, subsample, approx):
    img = image(52, 77, seed=3)
    base = decode(encode_baseline(img, Q_COARSE, subsample=subsample))
    prog = decode(encode_progressive(img, Q_COARSE, subsample=subsample, approx=approx))
    assert np.array_equal(prog, base)
    assert np.abs(base[..., :3] - img.astype(np.int64)).mean() < 12


def test_refuses_what_it_does_not_decode(lib):
    good = encode_baseline(image(16, 16), Q_FINE)
    assert gltf.decode_jpeg(good[:40]) is None          # truncated
    assert gltf.decode_jpeg(b"\x89PNG\r\n\x1a\n") is None
    arith = good.replace(b"\xff\xc0", b"\xff\xc9", 1)    # arithmetic-coded frame
    assert gltf.decode_jpeg(arith) is None
    assert b"JPEG" in A.load().rt_last_error()


def test_real_photographs(lib):
    """Two baseline photographs shipped with scikit-learn (when present): they decode, at their
    declared size, to a plausible natural image."""
    import importlib.util

    spec = importlib.util.find_spec("sklearn")
    if spec is None:
        pytest.skip("scikit-learn not installed")
    folder = Path(spec.origin).parent / "datasets" / "images"
    for name in ("china.jpg", "flower.jpg"):
        p = folder / name
        if not p.exists():
            pytest.skip(f"{name} not present")
        out = decode(p.read_bytes())
        assert out.shape == (427, 640, 4)
        rgb = out[..., :3].astype(np.float64)
        assert 20 < rgb.mean() < 235 and rgb.std() > 20
        # neighbouring pixels of a photograph are close on average (a decoding error breaks this)
        assert np.abs(np.diff(rgb, axis=1)).mean() < 20


def test_corrupted_streams_fail_cleanly(lib):
    """Seeded corruptions of valid baseline and progressive files (flipped bytes, truncations, spliced
    segments): every call returns an image or a refusal with a message; none crashes or hangs."""
    rng = np.random.default_rng(11)
    img = image(40, 56, seed=5)
    sources = [encode_baseline(img, Q_COARSE, subsample=True, restart=2),
               encode_progressive(img, Q_COARSE, subsample=True, approx=True)]
    decoded = refused = 0
    for src in sources:
        for trial in range(150):
            b = bytearray(src)
            kind = trial % 3
            if kind == 0:
                for _ in range(int(rng.integers(1, 8))):
                    b[int(rng.integers(2, len(b)))] = int(rng.integers(0, 256))
            elif kind == 1:
                b = b[: int(rng.integers(2, len(b)))]
            else:
                i, j = sorted(int(x) for x in rng.integers(2, len(b), 2))
                b = b[:i] + b[j:] + b[i:j]
            t = gltf.decode_jpeg(bytes(b))
            if t is None:
                refused += 1
                assert A.load().rt_last_error()
            else:
                decoded += 1
                assert np.isfinite(np.asarray(t.data)).all()
    assert decoded + refused == 2 * 150 and refused > 0
