"""Writes tests/golden/pyslfp_generalised_sle_lmax32.npz from the reference's fixtures.

Reads, from the reference's tests/data directory (the first argument, by
default the checkout this was made from):
  - pyslfp_love_numbers.txt: the Love-number table the reference's sea-level
    gate solves with (records radius, surface_gravity, axial h_c k_c m_u
    m_phi m_c, and a table of l with the twelve columns h_u l_u k_u h_phi
    l_phi k_phi h_v l_v k_v h_t l_t k_t; SI);
  - pyslfp_generalised_sea_level.txt: pyslfp's generalised sea-level solve
    at lmax 32 (scalar records inertia_moment, angular_momentum, omega;
    `field NAME` blocks of rows l m a b, the real orthonormal pyshtools
    coefficients without the Condon-Shortley phase, SI).
Keeps everything, the coefficients converted to the complex (l, m >= 0)
layout l(l+1)/2 + m with the Condon-Shortley phase that the library's
transforms use: c = a for m = 0, else (-1)^m (a - i b) / sqrt(2), as the
reference's tests/TestFixtures.cpp:79-110 reads them.

  python tests/golden/make_pyslfp_sle.py [reference tests/data directory]
"""

import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LMAX = 32
COLUMNS = ("h_u", "l_u", "k_u", "h_phi", "l_phi", "k_phi", "h_v", "l_v", "k_v", "h_t", "l_t", "k_t")


def love_table(path):
    out, rows, in_table = {}, [], False
    for line in path.read_text().splitlines():
        if not line or line.startswith("#"):
            continue
        parts = line.split()
        if in_table:
            rows.append([float(v) for v in parts])
            continue
        if parts[0] == "table":
            in_table = True
        elif parts[0] in ("radius", "surface_gravity"):
            out[parts[0]] = float(parts[1])
        elif parts[0] == "axial":
            out["axial"] = np.array([float(v) for v in parts[1:6]])  # h_c k_c m_u m_phi m_c
    table = np.array(rows)
    assert np.array_equal(table[:, 0], np.arange(table.shape[0])), "degrees 0, 1, 2, ... without gaps"
    for i, name in enumerate(COLUMNS):
        out["love_" + name] = table[:, 1 + i]
    return out


def sea_level_fixture(path):
    fields, scalars, current = {}, {}, None
    size = (LMAX + 1) * (LMAX + 2) // 2
    for line in path.read_text().splitlines():
        if not line or line.startswith("#"):
            continue
        parts = line.split()
        if not parts[0][0].isdigit():
            if parts[0] == "field":
                current = fields.setdefault(parts[1], np.zeros(size, dtype=np.complex128))
            else:
                scalars[parts[0]] = np.array([float(v) for v in parts[1:]])
                current = None
            continue
        l, m, a, b = int(parts[0]), int(parts[1]), float(parts[2]), float(parts[3])
        sign = -1.0 if m % 2 else 1.0
        current[l * (l + 1) // 2 + m] = a if m == 0 else sign * complex(a, -b) / np.sqrt(2.0)
    return fields, scalars


def main():
    data = pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/tests/data")
    love = love_table(data / "pyslfp_love_numbers.txt")
    fields, scalars = sea_level_fixture(data / "pyslfp_generalised_sea_level.txt")
    np.savez_compressed(HERE / "pyslfp_generalised_sle_lmax32.npz", **love,
                        **{"field_" + k: v for k, v in fields.items()},
                        **{"scalar_" + k: v for k, v in scalars.items()})
    print(f"{len(love['love_h_u'])} degrees of Love numbers; fields {sorted(fields)}; scalars {sorted(scalars)}")


if __name__ == "__main__":
    main()
