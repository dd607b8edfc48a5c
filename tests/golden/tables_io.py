"""Reader of the binary material-table dump written by the reference driver
(oracle/ref_recipe/ref_driver.cpp, "tables") and by the oracle (oracle_tables)."""
import numpy as np


def read_tables(path, n_materials=1):
    raw = open(path, "rb").read()
    off = 0
    out = []

    def take(n):
        nonlocal off
        a = np.frombuffer(raw, dtype="<f8", count=n, offset=off)
        off += 8 * n
        return a

    for _ in range(n_materials):
        nt = int(np.frombuffer(raw, dtype="<u8", count=1, offset=off)[0])
        off += 8
        temps = take(nt).copy()
        freq, vla, vta, dla, dta = (take(1000).copy() for _ in range(5))
        kinds = []
        for _k in range(3):
            sums = np.zeros(nt)
            tabs = np.zeros((nt, 1000, 2))
            for t in range(nt):
                sums[t] = take(1)[0]
                tabs[t] = take(2000).reshape(1000, 2)
            kinds.append((sums, tabs))
        out.append(dict(temps=temps, freq=freq, vel_la=vla, vel_ta=vta, dens_la=dla, dens_ta=dta,
                        base_sum=kinds[0][0], base=kinds[0][1], emit_sum=kinds[1][0], emit=kinds[1][1],
                        scatter_sum=kinds[2][0], scatter=kinds[2][1]))
    bounds = np.frombuffer(raw, dtype="<f8", count=2, offset=off).copy()
    return out, bounds
