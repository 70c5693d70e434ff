"""FITS input/output of the reference's data layout (Core/FitsIO.cs), host-side (no GPU).

Files are written here by an independent numpy writer (primary HDU, 80-character cards,
2880-byte blocks, big-endian data) in the layout FitsIO reads: uvw [bl][t][3], freq [ch],
vis [bl][t][ch][pol][2], flags [bl][t][ch][pol].  The readers must return what FitsIO returns:
v negated, (XX + YY) / norm from polarisations 0 and 3, flagged where the polarisation values
sum to non-zero, and the baseline-range overloads."""
import numpy as np
import pytest

from conftest import pkg


def _write_fits(path, arr, bitpix=-64, extra_cards=()):
    arr = np.asarray(arr)
    cards = [("SIMPLE", "T"), ("BITPIX", str(bitpix)), ("NAXIS", str(arr.ndim))]
    cards += [(f"NAXIS{i + 1}", str(n)) for i, n in enumerate(reversed(arr.shape))]
    cards += list(extra_cards)
    hdr = "".join(f"{k:<8}= {v:>20}".ljust(80) for k, v in cards) + "END".ljust(80)
    hdr = hdr.ljust((len(hdr) + 2879) // 2880 * 2880)
    data = arr.astype(">f8" if bitpix == -64 else ">f4").tobytes()
    data += b"\0" * ((-len(data)) % 2880)
    with open(path, "wb") as f:
        f.write(hdr.encode("ascii") + data)


def _read_fits(path):
    raw = open(path, "rb").read()
    cards = {}
    off = 0
    while True:
        card = raw[off:off + 80].decode("ascii")
        off += 80
        if card.startswith("END"):
            break
        if card[8:10] == "= ":
            cards[card[:8].strip()] = card[10:].split("/")[0].strip()
    off = (off + 2879) // 2880 * 2880
    shape = tuple(int(cards[f"NAXIS{i}"]) for i in range(int(cards["NAXIS"]), 0, -1))
    dt = ">f8" if cards["BITPIX"] == "-64" else ">f4"
    n = int(np.prod(shape))
    return cards, np.frombuffer(raw[off:off + n * np.dtype(dt).itemsize], dt).reshape(shape)


@pytest.fixture
def dataset(tmp_path):
    rng = np.random.default_rng(3)
    nbl, nt, nch, npol = 5, 7, 3, 4
    uvw = rng.standard_normal((nbl, nt, 3)) * 1000
    freq = np.linspace(1.2e9, 1.5e9, nch)
    vis = rng.standard_normal((nbl, nt, nch, npol, 2))
    flags = (rng.random((nbl, nt, nch, npol)) < 0.2).astype(np.float64)
    flags[0, 0, 0] = [1.0, -1.0, 0.0, 0.0]  # sums to zero: not flagged, as FitsIO decides
    paths = {k: tmp_path / f"{k}.fits" for k in ("uvw", "freq", "vis", "flags")}
    _write_fits(paths["uvw"], uvw, extra_cards=[("EXTEND", "T")])
    _write_fits(paths["freq"], freq)
    _write_fits(paths["vis"], vis)
    _write_fits(paths["flags"], flags)
    return dict(uvw=uvw, freq=freq, vis=vis, flags=flags, paths=paths, dims=(nbl, nt, nch))


def test_read_reference_layout(dataset):
    d, p = dataset, dataset["paths"]
    nbl, nt, nch = d["dims"]
    F = pkg.FitsIO
    assert F.CountBaselines(p["uvw"]) == nbl
    uvw = F.ReadUVW(p["uvw"])
    assert np.array_equal(uvw[..., 0], d["uvw"][..., 0]) and np.array_equal(uvw[..., 1], -d["uvw"][..., 1])
    assert np.array_equal(uvw[..., 2], d["uvw"][..., 2])
    assert np.array_equal(F.ReadUVW(p["uvw"], 1, 4), uvw[1:4])
    assert np.array_equal(F.ReadFrequencies(p["freq"]), d["freq"])
    norm = 2.0
    vis = F.ReadVisibilities(p["vis"], nbl, nt, nch, norm)
    expect = ((d["vis"][:, :, :, 0, 0] + d["vis"][:, :, :, 3, 0]) / norm
              + 1j * (d["vis"][:, :, :, 0, 1] + d["vis"][:, :, :, 3, 1]) / norm)
    assert np.array_equal(vis, expect)
    assert np.array_equal(F.ReadVisibilities(p["vis"], 4, nt, nch, norm, fromBl=2), expect[2:4])
    assert np.array_equal(F.ReadVisibilities(p["vis"], nbl, nt - 2, nch - 1, norm), expect[:, :nt - 2, :nch - 1])
    flags = F.ReadFlags(p["flags"], nbl, nt, nch)
    assert np.array_equal(flags, d["flags"].sum(axis=-1) != 0)
    assert not flags[0, 0, 0]
    assert np.array_equal(F.ReadFlags(p["flags"], 3, nt, nch, fromBl=1), flags[1:3])


def test_image_round_trip(tmp_path):
    rng = np.random.default_rng(8)
    img32 = rng.standard_normal((6, 9)).astype(np.float32)
    img64 = rng.standard_normal((5, 4))
    pkg.FitsIO.Write(img32, tmp_path / "a.fits")
    pkg.FitsIO.Write(img64, tmp_path / "b.fits")
    cards, raw = _read_fits(tmp_path / "a.fits")
    assert cards["SIMPLE"] == "T" and cards["BITPIX"] == "-32" and raw.shape == (6, 9)
    assert np.array_equal(raw.astype(np.float32), img32)
    assert np.array_equal(pkg.FitsIO.ReadImage(tmp_path / "a.fits"), img32)
    assert np.array_equal(pkg.FitsIO.ReadImageDouble(tmp_path / "b.fits"), img64)
    _write_fits(tmp_path / "c.fits", img64.astype(np.float32), bitpix=-32)
    assert np.array_equal(pkg.FitsIO.ReadImage(tmp_path / "c.fits"), img64.astype(np.float32))


def test_rejects_mismatched_files(tmp_path, dataset):
    p = dataset["paths"]
    with pytest.raises(pkg.P9IDGError):
        pkg.FitsIO.ReadUVW(p["vis"])  # wrong rank
    with pytest.raises(pkg.P9IDGError):
        pkg.FitsIO.ReadImage(p["freq"])
    with pytest.raises(pkg.P9IDGError):
        pkg.FitsIO.ReadUVW(p["uvw"], 2, 99)
    (tmp_path / "junk.fits").write_bytes(b"not a fits file" * 300)
    with pytest.raises(pkg.P9IDGError):
        pkg.FitsIO.ReadFrequencies(tmp_path / "junk.fits")
    (tmp_path / "short.fits").write_bytes(b"SIMPLE  =")
    with pytest.raises(pkg.P9IDGError):
        pkg.FitsIO.ReadFrequencies(tmp_path / "short.fits")
