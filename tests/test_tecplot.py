"""Tecplot output in the reference's format (input_output/visualization.f90), byte for byte.

The expected text below is written by hand from the reference's format statements
(write_headers :514-762, write_properties :1591-1716, write_df :920-1230) and gfortran's
edit descriptors: Ew.d as [-]0.<d digits>E<sign><2 digits> right-justified in w, Iw
right-justified, Aw of a blank-padded character(len=128) name cut to w characters, `(1x)`
ending each line with a blank. The distributions are chosen so that every written number is
exact, so the expected bytes follow from the formulas alone.
"""
import os

import numpy as np
import pytest

Z16 = "  0.0000000000000000E+00"   # E24.16 of 0
Z15 = "   0.000000000000000E+00"   # E24.15 of 0


def E16(v):
    return {0.0: Z16, 1.0: "  0.1000000000000000E+01", -1.0: " -0.1000000000000000E+01",
            2.0: "  0.2000000000000000E+01", -2.0: " -0.2000000000000000E+01",
            0.5: "  0.5000000000000000E+00", -0.5: " -0.5000000000000000E+00",
            0.25: "  0.2500000000000000E+00", 1.5: "  0.1500000000000000E+01",
            0.375: "  0.3750000000000000E+00", 32.0: "  0.3200000000000000E+02",
            "nan": "                     NaN"}[v]


def E15(v):
    return {0.0: Z15, 0.25: "   0.250000000000000E+00", 0.5: "   0.500000000000000E+00",
            0.75: "   0.750000000000000E+00", 1.0: "   0.100000000000000E+01",
            1.25: "   0.125000000000000E+01"}[v]


@pytest.fixture(scope="module")
def lib(pkg):
    if not os.path.exists(pkg.LIB_PATH):
        import importlib
        importlib.import_module("2d_dvm_microflows_gb300.build").build()
    return pkg.load_library()


@pytest.mark.parametrize("x,w,d,want", [
    (1.5, 24, 16, "  0.1500000000000000E+01"),
    (-1.5, 24, 16, " -0.1500000000000000E+01"),
    (0.0, 24, 15, "   0.000000000000000E+00"),
    (0.1, 24, 16, "  0.1000000000000000E+00"),
    (1.0e-120, 24, 16, "  0.1000000000000000-119"),   # three exponent digits: no E
    (-2.5e100, 24, 16, " -0.2500000000000000+101"),
    (123456.0, 24, 15, "   0.123456000000000E+06"),
    (2.0 / 3.0, 24, 16, "  0.6666666666666666E+00"),
    (float("nan"), 24, 16, "                     NaN"),
    (float("inf"), 24, 16, "                Infinity"),
])
def test_edit_descriptor(pkg, lib, x, w, d, want):
    assert pkg.fortran_e(x, w, d, lib=lib) == want


def _grid(pkg):
    a = np.array([-1.0, 0.0, 1.0])   # node volumes 1, 1, 1
    return pkg.physics.VelocityGrid(a, a.copy(), a.copy())


def _f():
    """Three cells on the 3^3 grid, l = i + 3 j + 9 k; (x, y, z) = (0, 0, 0) is l = 13."""
    f = np.zeros((3, 27))
    f[0, 12], f[0, 14] = 1.0, 1.0   # x = -1, +1: n 2, u 0, T 1 (mass 1.5)
    f[1, 13], f[1, 14] = 1.0, 1.0   # x = 0, +1: n 2, u 0.5, T 0.25
    f[2, 14] = 2.0                  # x = +1 only: n 2, u 1, T 0
    return f


PROPS = ("write_dens", "write_x_vel", "write_speed", "write_tr_temp", "write_rot_temp",
         "write_tot_temp", "write_temp_x", "write_tr_energy", "write_tot_energy",
         "write_entropy", "write_heat_flux_x", "write_pressure")


def test_properties_files(pkg, lib, tmp_path):
    base = str(tmp_path / "props")
    out = pkg.TecplotOutput(3, 1, 0.5, 1.0, mass=1.5, end_time=4, properties_filename=base,
                            properties=PROPS, properties_dump_freq=2, stress=(11, 12),
                            moments=(2,), lib=lib)
    out.write_headers()
    g, f = _grid(pkg), _f()
    out.write_properties(0.0, f=f, grid=g)
    out.write_properties(0.25, f=f, grid=g)

    names14 = ['"Density"     ', '"X-Velocity"  ', '"Speed"       ', '"Trans. Temp."',
               '"Rot. Temp."  ', '"Total Temp." ', '"Temp. X"     ', '"Trans. Energy',
               '"Total Energy"', '"Entropy"     ', '"Heat Flux X" ', '"Pressure"    ']
    head = ('title = "Macroscopic Properties"\n'
            'variables = "Time", "x-Location", "y-Location"' +
            "".join(" , " + n for n in names14) + ', "Tau 11", "Tau 12", "Moment  2" \n')
    # mixture rows: n, u, speed, T_tr, T_rot, T, Temp. X (zero in this file), E_tr, E,
    # entropy, q_x, p, tau_xx, tau_xy, the order-2 moment (zero in this file)
    ln2 = " -0.1386294361119891E+01"    # entropy of the third cell: -2 log 2
    mix = [(2.0, 0.0, 0.0, 1.0, 0.0, 1.0, 0.0, 1.5, 1.5, 0.0, 0.0, 1.0, -2.0, 0.0, 0.0),
           (2.0, 0.5, 0.5, 0.25, 0.0, 0.25, 0.0, 0.375, 0.375, 0.0, 0.0, 0.25, -0.5, 0.0, 0.0),
           (2.0, 1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, "ln2", 0.0, 0.0, 0.0, 0.0, 0.0)]
    xs = (0.25, 0.75, 1.25)

    def row(vals):
        return "".join(ln2 if v == "ln2" else E16(v) for v in vals)

    # compute_moment of order 2: (2+1)!! T^3.5 2^-1 normalises sum |c|^2 f times mass:
    # 1.5 * 2 / (2 * 1.5) = 1; 1.5 * 0.5 / (2 * 3 * 2^-8) = 32; at T = 0, 0 / 0

    want = head
    for t in (0.0, 0.25):
        want += "zone i=    3\n"
        for c in range(3):
            want += E15(t) + E15(xs[c]) + E15(0.5) + row(mix[c]) + " \n"
    assert open(base + ".dat").read() == want

    # the species file: trimmed names, locations from zero, Temp. X formed from f
    head1 = ('title = "Macroscopic Properties"\n'
             'variables = "Time", "x-Location", "y-Location", "Density", "X-Velocity", '
             '"Speed", "Trans. Temp.", "Rot. Temp.", "Total Temp.", "Temp. X", '
             '"Trans. Energy", "Total Energy", "Entropy", "Heat Flux X", "Pressure", '
             '"Tau 11", "Tau 12", "Moment  2" \n')
    spc = [(2.0, 0.0, 0.0, 1.0, 0.0, 1.0, 1.0, 1.5, 1.5, 0.0, 0.0, 1.0, -2.0, 0.0, 1.0),
           (2.0, 0.5, 0.5, 0.25, 0.0, 0.25, 0.25, 0.375, 0.375, 0.0, 0.0, 0.25, -0.5, 0.0,
            32.0),
           (2.0, 1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, "ln2", 0.0, 0.0, 0.0, 0.0, "nan")]
    want1 = head1
    for t in (0.0, 0.25):
        want1 += "zone i=    3\n"
        for c in range(3):
            want1 += E15(t) + E15((0.0, 0.5, 1.0)[c]) + E15(0.0) + row(spc[c]) + " \n"
    assert open(base + "_1.dat").read() == want1


def test_one_cell_zone_header(pkg, lib, tmp_path):
    """A one-cell run announces its zone length once, in the header: end_time / freq + 1
    outputs when freq divides end_time, + 2 otherwise."""
    for end, freq, n in ((4, 2, 3), (5, 2, 4)):
        base = str(tmp_path / ("one%d" % end))
        out = pkg.TecplotOutput(1, 1, 1.0, 1.0, end_time=end, properties_filename=base,
                                properties=("write_dens",), properties_dump_freq=freq, lib=lib)
        out.write_headers()
        lines = open(base + ".dat").read().split("\n")
        assert lines[2] == "zone i=%4d" % n
        out.write_properties(0.0, props=np.array([[2.0] + [0.0] * 19]))
        tail = open(base + ".dat").read().split("\n")[3]
        assert tail == Z15 + "   0.500000000000000E+00" + "   0.500000000000000E+00" + E16(2.0) + " "


def test_distribution_function_files(pkg, lib, tmp_path):
    """write_df at cell 3 in one and three dimensions: the third cell has no temperature,
    so its equilibrium is zero and the deviation column equals f."""
    g, f = _grid(pkg), _f()
    base = str(tmp_path / "df")
    out = pkg.TecplotOutput(3, 1, 0.5, 1.0, mass=1.5, df_filename=base, df_locations=[(3, 1)],
                            df_dimension=1, rot_levels=2, lib=lib)
    out.write_headers()
    out.write_df(0.0, f, g)
    want = ('title = "Distribution Function"\n'
            'variables = "X-Velocity", "Beta3", "Time", "Vel DistFunc", "Deviation", '
            '"Rot   1", "Rot   2", "Rot Energy" \n'
            'zone i=   3\n')
    for i, x in enumerate((-1.0, 0.0, 1.0)):
        fv = 2.0 if i == 2 else 0.0
        want += E16(x) + E16(1.0) + Z16 + E16(fv) + E16(fv) + Z16 * 3 + " \n"
    assert open(base + "_1_3_1.dat").read() == want

    base3 = str(tmp_path / "df3")
    out3 = pkg.TecplotOutput(3, 1, 0.5, 1.0, mass=1.5, df_filename=base3,
                             df_locations=[(3, 1)], df_dimension=3, lib=lib)
    out3.write_headers()
    out3.write_df(0.5, f, g)
    lines = open(base3 + "_1_3_1.dat").read().split("\n")
    assert lines[1] == ('variables = "X-Velocity", "Y-Velocity", "Z-Velocity", "Beta3", '
                        '"Time", "Vel DistFunc", "Deviation" ')
    assert lines[2] == "zone i=   3     , j=   3     , k=   3"
    rows = lines[3:3 + 27]
    v = (-1.0, 0.0, 1.0)
    for l, r in enumerate(rows):
        i, j, k = l % 3, (l // 3) % 3, l // 9
        fv = 2.0 if l == 14 else 0.0
        assert r == E16(v[i]) + E16(v[j]) + E16(v[k]) + E16(1.0) + E16(0.5) + E16(fv) + \
            E16(fv) + " "


def test_columns_from_phi_need_f(pkg, lib, tmp_path):
    out = pkg.TecplotOutput(2, 1, 1.0, 1.0, properties_filename=str(tmp_path / "p"),
                            properties=("write_entropy",), lib=lib)
    out.write_headers()
    with pytest.raises(pkg.DVMError):
        out.write_properties(0.0, props=np.zeros((2, 20)))
