"""Generate ``psi_json_ref.json``: parameter files in the reference's JSON form.

Encodes a small Psi and PsiDeep, as the reference's ``to_json`` builds them
(pyRBMonGPU/Psi.py:8-22, PsiDeep.py:8-24), with the reference's own ``NumpyEncoder``
(pyRBMonGPU/json_numpy.py, loaded by path: it needs only json and numpy).

    python tests/golden/make_json_golden.py [reference root]
"""
import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load(root):
    path = os.path.join(root, "pyRBMonGPU", "json_numpy.py")
    spec = importlib.util.spec_from_file_location("reference_json_numpy", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RBMONGPU_REF")
    if not root:
        sys.exit("usage: %s <RBMonGPU checkout>  (or set RBMONGPU_REF)" % sys.argv[0])
    jn = load(root)
    rng = np.random.default_rng(77)
    cn = lambda *s: rng.normal(size=s) + 1j * rng.normal(size=s)   # noqa: E731
    N, M = 4, 8
    psi = dict(type="Psi", alpha=np.zeros(N), beta=np.zeros(N), b=0.1 * cn(M), W=0.1 * cn(N, M), prefactor=0.75)
    conn0 = np.array([[0, 1, 2, 3, 0, 1], [1, 2, 3, 0, 1, 2]], dtype=np.uint32)
    conn1 = np.array([[0, 2, 4], [1, 3, 5]], dtype=np.uint32)
    deep = dict(type="PsiDeep", alpha=np.zeros(N), beta=np.zeros(N), b=[0.1 * cn(6), 0.1 * cn(3)],
                connections=[conn0, conn1], W=[0.1 * cn(2, 6), 0.1 * cn(2, 3)], final_weights=1.0 + 0.1 * cn(3),
                prefactor=1.0, free_quantum_axis=False)
    out = {name: json.loads(json.dumps(obj, cls=jn.NumpyEncoder)) for name, obj in (("psi", psi), ("deep", deep))}
    with open(os.path.join(HERE, "psi_json_ref.json"), "w") as f:
        json.dump(out, f)
    print("wrote psi_json_ref.json")


if __name__ == "__main__":
    main()
