"""JSON (de)serialisation of numpy arrays in the reference's checkpoint format
(pyANNonGPU/json_numpy.py:5-38): an array becomes
{"type": "ndarray", "dtype": ..., "complex": bool, "real"/"imag" | "data": nested lists}.
Kept identical so wavefunctions saved by either implementation load in the other."""

import json

import numpy as np


class NumpyEncoder(json.JSONEncoder):
    def default(self, obj):
        if isinstance(obj, np.ndarray):
            is_c = bool(np.iscomplexobj(obj))
            out = {"type": "ndarray", "dtype": str(obj.dtype), "complex": is_c}
            if is_c:
                out["real"] = obj.real.tolist()
                out["imag"] = obj.imag.tolist()
            else:
                out["data"] = obj.tolist()
            return out
        if isinstance(obj, np.generic):
            return obj.item()
        return super().default(obj)


class NumpyDecoder(json.JSONDecoder):
    def __init__(self, *args, **kwargs):
        super().__init__(*args, object_hook=self._hook, **kwargs)

    @staticmethod
    def _hook(obj):
        if obj.get("type") == "ndarray":
            dt = np.dtype(obj["dtype"])
            if obj["complex"]:
                return np.array(obj["real"], dtype=dt) + 1j * np.array(obj["imag"], dtype=dt)
            return np.array(obj["data"], dtype=dt)
        return obj
