"""The Lua 5.4 subset that runs scene scripts: number subtypes, operators, closures, varargs,
metatables, the libraries the scenes call, and error reporting."""
import math

import pytest

from em_lab_gb300.lua import Interpreter, LuaError, Xoshiro256


def run(src):
    out = []
    I = Interpreter(out=out.append)
    I.execute(src, "t.lua")
    return out


def ev(expr):
    return run(f"print({expr})")[0]


@pytest.mark.parametrize("expr,want", [
    ("3 / 2", "1.5"), ("7 // 2", "3"), ("-7 // 2", "-4"), ("7.5 // 2", "3.0"), ("7 % 3", "1"), ("-7 % 3", "2"),
    ("7 % -3", "-2"), ("5.5 % 2", "1.5"), ("2^10", "1024.0"), ("2^-1", "0.5"), ("-2^2", "-4.0"), ("1e3", "1000.0"),
    ("10 == 10.0", "true"), ("0.1 + 0.2", "0.3"), ("1/0", "inf"), ("-1/0", "-inf"), ("math.huge", "inf"),
    ("3 .. 4", "34"), ("1.0 .. ''", "1.0"), ("#'hello'", "5"), ("#{1, 2, 3, nil}", "3"), ("7 & 3", "3"),
    ("1 << 4", "16"), ("~0", "-1"), ("'10' + 1", "11"), ("math.floor(3.7)", "3"), ("math.ceil(-3.2)", "-3"),
    ("math.max(1, 2.5)", "2.5"), ("math.type(2)", "integer"), ("math.type(2.0)", "float"),
    ("math.tointeger(3.0)", "3"), ("tostring(1e100)", "1e+100"), ("tostring(-0.0)", "-0.0"),
    ("tonumber('0x1F')", "31"), ("tonumber(' 12.5 ')", "12.5"), ("tonumber('z')", "nil"),
    ("tonumber('ff', 16)", "255"), ("select('#', 1, nil, 3)", "3"), ("select(-1, 'a', 'b')", "b"),
    ("string.format('%5.2f|%d|%s|%g|%x|%q', 3.14159, 42, 'hi', 0.0001, 255, 'a\"b')", ' 3.14|42|hi|0.0001|ff|"a\\"b"'),
    ("string.format('%d', 3.0)", "3"), ("('abc'):upper()", "ABC"), ("('x'):rep(3, ',')", "x,x,x"),
    ("('hello'):sub(2, -2)", "ell"), ("('a,b,c'):find(',', 1, true)", "2\t2"), ("('key=val'):match('(%w+)=(%w+)')", "key\tval"),
    ("('hello world'):gsub('o', '0')", "hell0 w0rld\t2"), ("table.concat({1, 2, 3}, '-')", "1-2-3"),
    ("not nil", "true"), ("nil and 1", "nil"), ("false or 'x'", "x"), ("1 < 2 and 'a' < 'b'", "true"),
])
def test_expressions(expr, want):
    assert ev(expr) == want


def test_statements_closures_and_varargs():
    out = run("""
        local function fib(n) if n < 2 then return n end return fib(n - 1) + fib(n - 2) end
        local fs = {}
        for i = 1, 3 do fs[i] = function() return i end end
        local s = 0
        for i = 10, 1, -3 do s = s + i end
        local i = 0
        while true do i = i + 1; if i == 4 then break end end
        repeat i = i + 1; local z = i until z >= 7
        local function va(...) return select('#', ...), ... end
        local t = {}
        for k, v in ipairs({'x', 'y'}) do t[#t + 1] = k .. v end
        local n = 0
        for k, v in pairs({a = 1, b = 2, 3}) do n = n + 1 end
        local a, b, c = (function() return 1, 2 end)()
        print(fib(15), fs[1](), fs[3](), s, i, table.concat(t, ' '), n, a, b, c)
        print(va(nil, 2))
        print((va(1, 2)))
    """)
    assert out == ["610\t1\t3\t22\t7\t1x 2y\t3\t1\t2\tnil", "2\tnil\t2", "2"]


def test_metatables():
    out = run("""
        local V = {}
        V.__index = V
        V.__add = function(a, b) return setmetatable({v = a.v + b.v}, V) end
        V.__eq = function(a, b) return a.v == b.v end
        V.__lt = function(a, b) return a.v < b.v end
        V.__le = function(a, b) return a.v <= b.v end
        V.__len = function(a) return 99 end
        V.__call = function(self, x) return self.v * x end
        V.__tostring = function(a) return 'V(' .. a.v .. ')' end
        V.__concat = function(a, b) return tostring(a) .. '|' .. tostring(b) end
        V.__unm = function(a) return setmetatable({v = -a.v}, V) end
        function V:double() return self.v * 2 end
        local a, b = setmetatable({v = 1}, V), setmetatable({v = 2}, V)
        local logged = {}
        local proxy = setmetatable({}, {__newindex = function(t, k, v) rawset(t, k, v * 10) end})
        proxy.x = 4
        print(tostring(a + b), a == setmetatable({v = 1}, V), a < b, b <= a, #a, a(5), a:double(), a .. b, tostring(-b))
        print(proxy.x, rawget(proxy, 'x'), getmetatable(a) == V)
    """)
    assert out == ["V(3)\ttrue\ttrue\tfalse\t99\t5\t2\tV(1)|V(2)\tV(-2)", "40\t40\ttrue"]


def test_errors_are_lua_errors():
    out = run("""
        print(pcall(function() error('boom') end))
        print(pcall(function() local x = nil; return x.y end))
        print(pcall(function() return 1 + {} end))
        print(pcall(error, {code = 7}))
    """)
    assert out[0] == "false\tboom"
    assert out[1].startswith("false\t") and "index a nil value" in out[1]
    assert "arithmetic on a table value" in out[2]
    assert out[3].startswith("false\ttable:")
    with pytest.raises(LuaError, match="t.lua:1:"):
        run("local x = = 1")
    with pytest.raises(LuaError, match="goto"):
        run("goto done")


def test_xoshiro_reference_sequence_and_lua_projection():
    x = Xoshiro256()
    x.s = [1, 2, 3, 4]
    assert [x.next() for _ in range(4)] == [11520, 0, 1509978240, 1215971899390074240]
    out = run("math.randomseed(42); local a = {} for i = 1, 200 do a[i] = math.random(1, 6) end "
              "math.randomseed(42); local same = true for i = 1, 200 do same = same and a[i] == math.random(1, 6) end "
              "local lo, hi = 7, 0 for i = 1, 200 do lo = math.min(lo, a[i]); hi = math.max(hi, a[i]) end "
              "local f = math.random() print(same, lo, hi, f >= 0 and f < 1, math.type(a[1]))")
    assert out == ["true\t1\t6\ttrue\tinteger"]


def test_math_matches_python():
    out = run("print(math.sqrt(2), math.sin(1), math.atan(1, 2), math.log(8, 2), math.exp(1), math.fmod(7, 3), "
              "math.rad(180), math.deg(math.pi))")
    vals = [float(v) for v in out[0].split("\t")]
    want = [math.sqrt(2), math.sin(1), math.atan2(1, 2), 3.0, math.e, 1.0, math.pi, 180.0]
    for got, w in zip(vals, want):
        assert abs(got - w) <= 1e-13 * max(1.0, abs(w))
