"""Launch autotuner with a JSON result cache.

``UCFDFlowSysAutotune`` (native, flowsys.cpp) times every launch candidate
of the sweeps on the system at hand -- threads per block x block-sweep
variant for block LU-SGS, threads per block x {CUDA graph, persistent
kernel} for the scalar LU-SGS loop -- and keeps the fastest.  No candidate
changes a result; they differ only in speed.

The cache is one JSON object per file, keyed by
``"<gpu name>|<sms> SMs|<kind>|N=<cells>|nface=<faces>|nvars=<nvars>|prec=<precision>"``,
so a tuned choice is reused for the same mesh size on the same GPU model.
The default file is ``$UCFD_AUTOTUNE_CACHE`` or
``~/.cache/ucfd_gb300/autotune.json``.
"""
from __future__ import annotations

import json
import os
import tempfile
from ctypes import byref, c_int, create_string_buffer

from .lib import LaunchConfig, call

PRECISION_NAMES = {0: "fp64", 1: "fp64_fma", 2: "fp32"}


def default_path() -> str:
    env = os.environ.get("UCFD_AUTOTUNE_CACHE")
    if env:
        return env
    return os.path.join(os.path.expanduser("~"), ".cache", "ucfd_gb300", "autotune.json")


def device_key() -> str:
    name = create_string_buffer(256)
    sms = c_int()
    call("UCFDDeviceInfo", name, 256, byref(sms))
    return f"{name.value.decode(errors='replace')}|{sms.value} SMs"


def cache_key(sys) -> str:
    if sys.kind is None:
        raise ValueError("autotune needs set_lusgs or set_blusgs first")
    prec = PRECISION_NAMES.get(sys.precision, str(sys.precision))
    return f"{device_key()}|{sys.kind}|N={sys.nlocal}|nface={sys.nfaces}|nvars={sys.nvars}|prec={prec}"


def load_cache(path: str) -> dict:
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def store_cache(path: str, data: dict) -> None:
    """Writes the whole cache atomically (temporary file + rename)."""
    d = os.path.dirname(os.path.abspath(path))
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(prefix=".autotune.", dir=d)
    try:
        with os.fdopen(fd, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except BaseException:
        try:
            os.unlink(tmp)
        except OSError:
            pass
        raise


def valid_entry(e) -> bool:
    return (isinstance(e, dict) and e.get("threads_per_block") in (0, 32, 64, 96, 128, 160, 192, 224, 256)
            and e.get("sweep_variant") in (0, 1, 2, 3, 4) and e.get("run_mode") in (0, 1))


def tune(sys, reps: int = 5, cache: str | bool | None = None, force: bool = False) -> dict:
    """Applies the cached launch choice for ``sys`` or measures and stores one.

    Returns the chosen configuration with ``"source"`` = ``"cache"`` or
    ``"measured"``.
    """
    path = None
    if cache is True:
        path = default_path()
    elif isinstance(cache, str):
        path = cache
    key = cache_key(sys) if path else None
    if path and not force:
        entry = load_cache(path).get(key)
        if valid_entry(entry):
            sys.set_launch_config(**entry)
            out = sys.launch_config()
            out["ms"] = entry.get("ms", 0.0)
            out["source"] = "cache"
            return out
    cfg = LaunchConfig()
    call("UCFDFlowSysAutotune", sys._h, reps, byref(cfg))
    out = cfg.as_dict()
    if path:
        data = load_cache(path)
        data[key] = dict(out)
        store_cache(path, data)
    out["source"] = "measured"
    return out
