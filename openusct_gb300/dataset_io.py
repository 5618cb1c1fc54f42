"""Acquisition files: the Dataset HDF5 layout and the UARP/UDSP v4.0 Set.

``save`` / ``load`` write and read the platform's Dataset file
(simulation/ringfwi/dataset.py:112-174; the layout is specified in
software/schema/README.md): root attributes ``format_version``, ``description``
and ``created_by``; ``/geometry`` with ``n_elements``, ``radius_m``,
``centre_freq_hz``, ``array_type`` and ``element_pos[N, dim]``;
``/acquisition`` with ``sample_rate_hz``, ``tx_centre_freq_hz``,
``nominal_speed_m_s``, ``data`` (FP32 ``[n_tx, n_samples, n_rx]``, gzip),
``tx_wavelet`` and ``tx_elements``; optional ``/ground_truth`` with ``h_m``
and ``c`` (gzip).  A file whose ``format_version`` has another major version
is refused, as the schema asks of readers.

``to_uarp_set`` / ``from_uarp_set`` write and read the UDSP v4.0 Set of the
UARP toolbox (simulation/ringfwi/uarp_format.py:37-116): ``/Series/Series000``
with ``Dimensions`` (``Value``; ``Dimension1`` fast time, uniform; ``Dimension2``
receive elements, ``Sparse.Points``) and ``Frames`` (one FP32 ``[nt, n_rx]``
frame per transmit, ``Description = "tx_element=<i>"``).

Files go through :mod:`openusct_gb300.hdf5` (no h5py needed).  The functions
take the reference's ``Dataset`` or this package's equivalent
(:mod:`openusct_gb300.acquire`), and the readers return the reference's class
when ``ringfwi`` is importable.
"""

from __future__ import annotations

import numpy as np

from . import hdf5

FORMAT_VERSION = "1.0"
UARP_SCHEMA_VERSION = "4.0"


def _classes():
    from .acquire import _classes as c
    return c()


def _text(v) -> str:
    """An attribute as text: variable-length strings come back as str,
    fixed-length ones as bytes."""
    if isinstance(v, (bytes, np.bytes_)):
        return bytes(v).decode("utf-8", "replace").rstrip("\0")
    return str(v)


def _put_attrs(obj, pairs):
    for k, v in pairs:
        obj.attrs[k] = v


# ---------------------------------------------------------------------------
# the Dataset file
# ---------------------------------------------------------------------------
def save(ds, path, compression="gzip"):
    """Write ``ds`` as a Dataset file (Dataset.save, dataset.py:112-140)."""
    meta = getattr(ds, "metadata", None) or {}
    geo = ds.geometry
    with hdf5.File(path, "w") as f:
        _put_attrs(f, (("format_version", FORMAT_VERSION),
                       ("description", str(meta.get("description", ""))),
                       ("created_by", str(meta.get("created_by", "OpenUSCT")))))
        g = f.create_group("geometry")
        _put_attrs(g, (("n_elements", int(geo.n_elements)), ("radius_m", float(geo.radius_m)),
                       ("centre_freq_hz", float(geo.centre_freq_hz)),
                       ("array_type", str(geo.array_type))))
        g.create_dataset("element_pos", data=np.asarray(geo.element_pos))
        a = f.create_group("acquisition")
        _put_attrs(a, (("sample_rate_hz", float(ds.sample_rate_hz)),
                       ("tx_centre_freq_hz", float(ds.tx_centre_freq_hz)),
                       ("nominal_speed_m_s", float(ds.nominal_speed_m_s))))
        a.create_dataset("data", data=np.asarray(ds.data, dtype=np.float32), compression=compression)
        a.create_dataset("tx_wavelet", data=np.asarray(ds.tx_wavelet))
        a.create_dataset("tx_elements", data=np.asarray(ds.tx_elements))
        if ds.ground_truth is not None:
            t = f.create_group("ground_truth")
            t.attrs["h_m"] = float(ds.ground_truth["h_m"])
            t.create_dataset("c", data=np.asarray(ds.ground_truth["c"]), compression=compression)


def _check_version(v):
    if v is None:
        return
    major = _text(v).split(".")[0]
    if major != FORMAT_VERSION.split(".")[0]:
        raise ValueError(f"Dataset format_version {_text(v)!r}: this reader knows major version "
                         f"{FORMAT_VERSION.split('.')[0]}")


def load(path):
    """Read a Dataset file (Dataset.load, dataset.py:142-174)."""
    RG, RD = _classes()
    with hdf5.File(path, "r") as f:
        _check_version(f.attrs.get("format_version"))
        g, a = f["geometry"], f["acquisition"]
        geom = RG(element_pos=g["element_pos"][()], radius_m=float(g.attrs["radius_m"]),
                  centre_freq_hz=float(g.attrs["centre_freq_hz"]),
                  array_type=_text(g.attrs["array_type"]))
        truth = None
        if "ground_truth" in f:
            t = f["ground_truth"]
            truth = {"c": t["c"][()], "h_m": float(t.attrs["h_m"])}
        meta = {k: _text(f.attrs.get(k, "")) for k in ("description", "created_by",
                                                         "format_version")}
        return RD(geometry=geom, data=a["data"][()], sample_rate_hz=float(a.attrs["sample_rate_hz"]),
                  tx_wavelet=a["tx_wavelet"][()],
                  tx_centre_freq_hz=float(a.attrs["tx_centre_freq_hz"]),
                  nominal_speed_m_s=float(a.attrs["nominal_speed_m_s"]),
                  tx_elements=a["tx_elements"][()] if "tx_elements" in a else None,
                  ground_truth=truth, metadata=meta)


# ---------------------------------------------------------------------------
# the UARP / UDSP v4.0 Set
# ---------------------------------------------------------------------------
# (path under Series000, attributes) of the Set's descriptive groups
_UDSP_QUANTITIES = (
    ("Dimensions/Value", (("Description", "Signal amplitude"), ("Unit", "Amplitude"),
                          ("Scale", "None"))),
    ("Dimensions/Dimension1/DimensionQuantity", (("Description", "Time"), ("Unit", "Seconds"),
                                                 ("Scale", "None"))),
    ("Dimensions/Dimension2/DimensionQuantity", (("Description", "Element position"),
                                                 ("Unit", "Metres"), ("Scale", "None"))),
)
_FRAME = "Frame%06d"
_TX_TAG = "tx_element="


def to_uarp_set(ds, path, description="OpenUSCT full-matrix-capture acquisition",
                timestamp="1970-01-01T00:00:00", compression="gzip"):
    """Write ``ds`` as a UDSP v4.0 Set (uarp_format.py:37-81)."""
    tx = np.asarray(ds.tx_elements)
    data = np.asarray(ds.data)
    with hdf5.File(path, "w") as f:
        _put_attrs(f, (("Version", UARP_SCHEMA_VERSION), ("Timestamp", timestamp),
                       ("Description", description)))
        s = f.create_group("Series/Series000")
        _put_attrs(s, (("Description", "Full-matrix capture channel data"),
                       ("State", "Analytical" if ds.ground_truth is not None else "Measured"),
                       ("Platform", "OpenUSCT"), ("Source", "Simulator")))
        for sub, attrs in _UDSP_QUANTITIES:
            _put_attrs(s.create_group(sub), attrs)
        d1 = s["Dimensions/Dimension1"]
        _put_attrs(d1, (("Description", "Fast time"), ("Uniform.Size", int(data.shape[1])),
                        ("Uniform.Stride", float(1.0 / ds.sample_rate_hz)),
                        ("Uniform.Offset", 0.0)))
        d2 = s["Dimensions/Dimension2"]
        d2.attrs["Description"] = "Receive element"
        d2.create_dataset("Sparse.Points", data=np.asarray(ds.geometry.element_pos))
        fr = s.create_group("Frames")
        fr.attrs["Size"] = int(data.shape[0])
        for i in range(data.shape[0]):
            one = fr.create_dataset(_FRAME % i, data=data[i].astype(np.float32),
                                    compression=compression)
            _put_attrs(one, (("Description", f"{_TX_TAG}{int(tx[i])}"), ("Delay", 0.0)))


def from_uarp_set(path, nominal_speed_m_s=1500.0):
    """Read a UDSP v4.0 Set into a Dataset (uarp_format.py:84-116): the frames
    in name order, each transmit's element from its description (its index
    when the description names none), the radius as the largest element
    distance from the centre; no wavelet, centre frequency or ground truth
    (a Set does not carry them)."""
    RG, RD = _classes()
    with hdf5.File(path, "r") as f:
        s = f["Series/Series000"]
        d1 = s["Dimensions/Dimension1"]
        nt = int(d1.attrs["Uniform.Size"])
        dt = float(d1.attrs["Uniform.Stride"])
        pos = s["Dimensions/Dimension2/Sparse.Points"][()]
        fr = s["Frames"]
        names = sorted(k for k in fr.keys() if k.startswith("Frame"))
        frames, tx = [], []
        for i, k in enumerate(names):
            ds_k = fr[k]
            frames.append(ds_k[()])
            desc = _text(ds_k.attrs.get("Description", ""))
            tx.append(int(desc.split("=", 1)[1]) if "=" in desc else i)
    data = np.stack(frames) if frames else np.zeros((0, nt, len(pos)), np.float32)
    radius = float(np.linalg.norm(pos, axis=1).max()) if len(pos) else 0.0
    geom = RG(element_pos=pos, radius_m=radius, centre_freq_hz=0.0,
              array_type="cylinder" if pos.shape[1] == 3 else "ring")
    return RD(geometry=geom, data=data, sample_rate_hz=1.0 / dt, tx_wavelet=np.zeros(nt),
              tx_centre_freq_hz=0.0, nominal_speed_m_s=nominal_speed_m_s,
              tx_elements=np.asarray(tx), ground_truth=None)
