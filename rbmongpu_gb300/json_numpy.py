"""JSON encoding of numpy arrays in the reference's on-disk format
(pyRBMonGPU/json_numpy.py:5-36): an array becomes {"type": "ndarray", "dtype": ...,
"complex": bool} with "data", or "real" and "imag" lists for complex arrays, so that
parameter files written by either implementation load in the other."""
import json

import numpy as np


class NumpyEncoder(json.JSONEncoder):
    def default(self, obj):
        if isinstance(obj, np.ndarray):
            out = {"type": "ndarray", "dtype": str(obj.dtype), "complex": bool(np.iscomplexobj(obj))}
            if out["complex"]:
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
        super().__init__(*args, object_hook=self.object_hook, **kwargs)

    @staticmethod
    def object_hook(obj):
        if obj.get("type") == "ndarray":
            dtype = np.dtype(obj["dtype"])
            if obj["complex"]:
                return np.array(obj["real"], dtype=dtype) + 1j * np.array(obj["imag"], dtype=dtype)
            return np.array(obj["data"], dtype=dtype)
        return obj


def encode(obj):
    """obj with its arrays in the JSON form (a plain JSON-compatible structure)."""
    return json.loads(json.dumps(obj, cls=NumpyEncoder))


def decode(obj):
    """The inverse of encode: the JSON form with its arrays as numpy arrays."""
    return json.loads(json.dumps(obj), cls=NumpyDecoder)
