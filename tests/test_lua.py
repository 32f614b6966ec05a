"""The Lua subset that runs scripted symmetries (dpx.lua), on the CPU: the
language pieces scripts use, Populate's contract as the reference's
LuaSymmetry::PreCalculate calls it (Backend/Backend/Symmetry.cpp:463-521),
the reference's own Cartesian-lattice script from its scripted goldens, and
a scripted symmetry decoded from a state into ManualSymmetry rows."""
import gzip
import json
import math
import os

import numpy as np
import pytest

from dpx import lua
from dpx import models as M
from dpx import state as S

GOLD = os.path.join(os.path.dirname(__file__), "golden", "scripted.json.gz")


def _run(src):
    L = lua.Interpreter()
    L.run(src)
    return L.G.get


def test_expressions_and_precedence():
    g = _run("""
        a = 2 + 3 * 4 ^ 2 / 8 - -1     -- ^ binds tighter than unary minus and *
        b = -2 ^ 2                      -- -(2^2)
        c = 2 ^ 3 ^ 2                   -- right associative
        d = 7 % 3 + (-7) % 3 + 7.5 % -2
        e = 1 .. 2 .. "x" .. 1.5
        f = not nil and 3 or 4
        g = nil or false
        h = 1 < 2 and "lt" or "ge"
        i = "a" < "b" and 10 == 10.0 and "1" ~= 1
        j = #"hello" + #{1, 2, 3, nil}
        k = 10 / 4
        l = 1 / 0 > 1e308
    """)
    assert g("a") == 2 + 3 * 16 / 8 + 1
    assert g("b") == -4 and g("c") == 512
    assert g("d") == 1 + 2 + (-0.5)
    assert g("e") == "12x1.5"
    assert g("f") == 3 and g("g") is False and g("h") == "lt" and g("i") is True
    assert g("j") == 8 and g("k") == 2.5 and g("l") is True


def test_statements_tables_and_closures():
    g = _run("""
        local function fib(n) if n < 2 then return n end return fib(n - 1) + fib(n - 2) end
        f10 = fib(10)
        t = {}
        for i = 10, 1, -3 do t[#t + 1] = i end
        s = table.concat(t, ",")
        local acc = 0
        for _, v in ipairs({5, 6, 7}) do acc = acc + v end
        sum = acc
        cnt = 0
        for k, v in pairs({x = 1, y = 2, 3}) do cnt = cnt + v end
        function counter() local c = 0; return function() c = c + 1; return c end end
        local nx = counter(); nx(); nx()
        three = nx()
        w = 0
        while true do w = w + 1; if w >= 5 then break end end
        repeat w = w - 2 until w < 0
        obj = {v = 3}
        function obj:twice() return 2 * self.v end
        tw = obj:twice()
        q, r = (function(...) return select("#", ...), ... end)(7, 8)
        fmt = string.format("%d|%.3f|%5s|%x", 42, math.pi, "ab", 255)
        up = ("abc"):upper() .. string.sub("hello", 2, -2)
        tn = tonumber("0x10") + tonumber(" 2.5 ")
        m = math.max(1, 9, 4) + math.floor(-1.5) + math.sqrt(16)
    """)
    assert g("f10") == 55 and g("s") == "10,7,4,1" and g("sum") == 18 and g("cnt") == 6
    assert g("three") == 3 and g("w") == -1 and g("tw") == 6
    assert g("q") == 2 and g("r") == 7
    assert g("fmt") == "42|3.142|   ab|ff" and g("up") == "ABCell" and g("tn") == 18.5 and g("m") == 11


def test_errors_and_budget():
    with pytest.raises(lua.LuaError, match="bad parameters"):
        _run('error("bad parameters")')
    with pytest.raises(lua.LuaError):
        _run("x = nil + 1")
    with pytest.raises(lua.LuaError):
        _run("x = {} .. 'a'")
    with pytest.raises(lua.LuaError):
        _run("for i = 1 do end")
    L = lua.Interpreter(max_steps=10_000)
    with pytest.raises(lua.LuaError, match="budget"):
        L.run("while true do end")
    L = lua.Interpreter()
    assert L.G.get("os") is None and L.G.get("io") is None and L.G.get("load") is None


HELIX = """
Information = {Name = "helix", Type = "Symmetry", NLP = 3, MinLayers = 1, MaxLayers = 1}
function Populate(p, nlayers)
    if p == nil or nlayers ~= 1 or table.getn(p[1]) ~= 3 then
        error("parameter matrix must be 1x3")
    end
    local radius, pitch, n = p[1][1], p[1][2], p[1][3]
    local res = {}
    for k = 0, n - 1 do
        local phi = 2 * math.pi * k / 13
        res[k + 1] = {radius * math.cos(phi), radius * math.sin(phi), pitch * k / 13, 0, 0, math.deg(phi)}
    end
    return res
end
"""


def test_populate_contract():
    rows = lua.populate(HELIX, [[12.0, 8.0, 26]])
    k = np.arange(26)
    phi = 2 * np.pi * k / 13
    want = np.stack([12 * np.cos(phi), 12 * np.sin(phi), 8.0 * k / 13, 0 * k, 0 * k, np.degrees(phi)], axis=1)
    assert rows.shape == (26, 6) and np.allclose(rows, want, rtol=0, atol=1e-12)
    with pytest.raises(lua.LuaError, match="1x3"):
        lua.populate(HELIX, [[12.0, 8.0]])
    # rows shorter than six or with non-numbers read as 0 (getlocrot, Symmetry.cpp:441-461)
    short = 'Information = {}\nfunction Populate(p, n) return {{1, 2}, {3, "x", 4}} end'
    assert np.array_equal(lua.populate(short, [[0]]), [[1, 2, 0, 0, 0, 0], [3, 0, 4, 0, 0, 0]])
    with pytest.raises(lua.LuaError):
        lua.populate("function Populate(p, n) return {} end", [[0]])  # no Information table


def test_reference_cartesian_script():
    """The reference's "Space filling symmetry - Cartesian" script (its scripted
    goldens' symmetry) with those goldens' parameters: 3 x 2 x 3 copies, 4, 4
    and 8.13 nm apart, x outermost."""
    with gzip.open(GOLD, "rt") as f:
        data = json.load(f)
    case = next(iter(data["cases"].values()))
    node = case["state"]["Domain"]["Populations"][0]["Models"][0]
    assert node["Type"] == "Scripted Symmetry"
    rows = lua.populate(data["script"], node["Parameters"], node["nLayers"])
    want = [[x * 4.0, y * 4.0, z * 8.13, 0, 0, 0] for x in range(3) for y in range(2) for z in range(3)]
    assert np.allclose(rows, want, rtol=0, atol=1e-12)
    with pytest.raises(lua.LuaError, match="6x1"):
        lua.populate(data["script"], node["Parameters"][:4], 4)


def test_scripted_symmetry_state_decodes_to_rows(tmp_path):
    """A scripted symmetry in a state becomes a ManualSymmetry of the script's
    rows, composed like a manual one (here over a PDB leaf, hybrid path)."""
    p = tmp_path / "sub.pdb"
    p.write_text("ATOM      1  C   ALA A   1       0.000   0.000   0.000  1.00  0.00           C\n"
                 "ATOM      2  O   ALA A   1       1.200   0.000   0.000  1.00  0.00           O\nEND\n")
    leaf = {"Type": "PDB", "Filename": "C:\\x\\sub.pdb", "Centered": False, "Use_Grid": True,
            "ExtraParameters": [1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0],
            "Location": {"x": 0, "y": 0, "z": 0, "alpha": 0, "beta": 0, "gamma": 0}}
    node = {"Type": "Scripted Symmetry", "Filename": "D:\\scripts\\helix.lua", "Parameters": [[12.0, 8.0, 5]],
            "nLayers": 1, "nlp": 3, "ExtraParameters": [2.0], "Use_Grid": False, "Children": [leaf],
            "Location": {"x": 0, "y": 0, "z": 0, "alpha": 0, "beta": 0, "gamma": 0}}
    state = {"DomainPreferences": {"GridSize": 24, "qMax": 4.0, "OrientationMethod": "Monte Carlo (Mersenne Twister)",
                                   "OrientationIterations": 1000, "Convergence": 0.001, "UseGrid": True},
             "Domain": {"Scale": 1.0, "Constant": 0.0, "Populations": [{"PopulationSize": 1.0, "Models": [node]}]}}
    job = S.decode(state, base_dir=str(tmp_path), files={"helix.lua": HELIX})
    (w, amps), = job.populations
    ms, = amps
    assert isinstance(ms, M.ManualSymmetry) and not ms.use_grid and abs(ms.scale - 2.0) < 1e-15
    want = lua.populate(HELIX, [[12.0, 8.0, 5]])
    assert np.allclose(ms.trans, want[:, :3], atol=1e-12)
    for ang, row in zip(ms.rot, want):  # the same rotations (the angles may come back as another triple)
        assert np.allclose(S._euler_matrix(*ang), S._euler_matrix(*np.radians(row[3:6])), atol=1e-12)
