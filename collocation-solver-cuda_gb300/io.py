"""Solution files in the reference's text format (BVPDAEReadWriteData.py:13-96).

Layout, one item per line unless noted:

    nt:
    <N>
    t:
    <t_0> <t_1> ... <t_{N-1}>           (space separated, trailing space)
    ny:
    <n_y>
    y:
    <y_i0> ... <y_i(n_y-1)>             (N lines)
    nz:
    <n_z>
    z:
    <z_i0> ...                          (N lines)
    np:
    <n_p>
    p:
    <p_0> ...                           (no trailing newline)

Numbers are written with Python's str() of a float (shortest repr), as the
reference's '{}'.format does, so files written here are byte-identical to the
reference's for the same values.  Both functions return an error code (0 ok,
1 failure) instead of raising, like the reference.
"""
import numpy as np


def bvpdae_read_data(fname):
    """Returns (error, t0, y0, z0, p0); error = 1 and empty lists on failure."""
    try:
        with open(fname, "r") as f:
            lines = f.read().split("\n")
        pos = 0

        def nxt():
            nonlocal pos
            line = lines[pos]
            pos += 1
            return line

        nxt()
        N = int(nxt())
        nxt()
        t0 = np.array([float(v) for v in nxt().rstrip().split(" ")[:N]], dtype=np.float64)
        if t0.shape[0] != N:
            raise ValueError("short t line")
        nxt()
        ny = int(nxt())
        nxt()
        y0 = np.zeros((N, ny), dtype=np.float64)
        for i in range(N):
            vals = nxt().rstrip().split(" ")
            for j in range(ny):
                y0[i, j] = float(vals[j])
        nxt()
        nz = int(nxt())
        nxt()
        z0 = np.zeros((N, nz), dtype=np.float64)
        for i in range(N):
            vals = nxt().rstrip().split(" ")
            for j in range(nz):
                z0[i, j] = float(vals[j])
        nxt()
        npar = int(nxt())
        nxt()
        vals = nxt().rstrip().split(" ")
        p0 = np.zeros(npar, dtype=np.float64)
        for i in range(npar):
            p0[i] = float(vals[i])
        return 0, t0, y0, z0, p0
    except Exception:  # noqa: BLE001 - the reference reports any failure as error 1
        return 1, [], [], [], []


def _fmt(v):
    return "{}".format(float(v))


def bvpdae_write_data(fname, N, n_y, n_z, n_p, t_span, y0, z0, p0):
    """Write a solution file; returns 0 on success, 1 on failure."""
    try:
        parts = ["nt:\n{}\nt:\n".format(N)]
        parts.append("".join(_fmt(t_span[i]) + " " for i in range(N)))
        parts.append("\nny:\n{}\ny:\n".format(n_y))
        for i in range(N):
            parts.append("".join(_fmt(y0[i, j]) + " " for j in range(n_y)) + "\n")
        parts.append("nz:\n{}\nz:\n".format(n_z))
        for i in range(N):
            parts.append("".join(_fmt(z0[i, j]) + " " for j in range(n_z)) + "\n")
        parts.append("np:\n{}\np:\n".format(n_p))
        parts.append("".join(_fmt(p0[i]) + " " for i in range(n_p)))
        with open(fname, "w") as f:
            f.write("".join(parts))
        return 0
    except Exception:  # noqa: BLE001
        return 1
