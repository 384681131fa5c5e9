"""Load/save helpers for the committed golden fixtures (one case per .npz)."""
import numpy as np


def save_case(path, kind, para, x, y, **extra):
    arrs = {f"para__{k}": np.asarray(v) for k, v in para.items()}
    np.savez_compressed(path, kind=np.array(kind), x=x, y=y, **arrs,
                        **{f"extra__{k}": np.asarray(v) for k, v in extra.items()})


def load_case(path):
    z = np.load(path, allow_pickle=False)
    para = {}
    for k in z.files:
        if k.startswith("para__"):
            v = z[k]
            para[k[6:]] = v[()] if v.ndim == 0 else v
    extra = {k[7:]: z[k] for k in z.files if k.startswith("extra__")}
    return dict(kind=str(z["kind"]), para=para, x=z["x"], y=z["y"], extra=extra)
