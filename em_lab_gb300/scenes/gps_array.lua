-- Adaptive GPS array: four dual-probe square patches (right-hand circular through a hybrid) keep a
-- satellite and null a jammer with MVDR weights.
local lambda = 24
local pml    = 10
scene { name = "Adaptive 2x2 patch array", size = {128, 128, 112}, pml = pml, wavelength = lambda }

local adapt  = param { name = "adapt", label = "adaptation", choices = {"ideal", "blind"} }
local jam_az = param { name = "jammer_azimuth", label = "jammer azimuth (deg)", default = 250, min = 0, max = 345, step = 15 }

local zg, h        = pml + 8, 3        -- ground plate, patch height (cells)
local d, side, pin = 13, 11, 2         -- spacing, patch side, probe inset (cells)
local c            = grid.center
local zt           = zg + h
local half         = d / 2 + side / 2 + 6
sheet { min = vec(c.x - half, c.y - half, zg), max = vec(c.x + half, c.y + half, zg) }

local elements = {}
local n = 0
for _, sy in ipairs({-1, 1}) do
  for _, sx in ipairs({-1, 1}) do
    n = n + 1
    local ex, ey = c.x + sx * d / 2, c.y + sy * d / 2
    local x0, y0 = ex - side / 2, ey - side / 2
    sheet { min = vec(x0, y0, zt), max = vec(x0 + side, y0 + side, zt) }
    monopole { base = vec(x0 + pin, ey, zg), orientation = "+z", length = h, amplitude = 1, name = "P" .. n .. "x" }
    monopole { base = vec(ex, y0 + pin, zg), orientation = "+z", length = h, amplitude = 1, name = "P" .. n .. "y" }
    elements[n] = { x = "P" .. n .. "x", y = "P" .. n .. "y", center = vec(ex, ey, zt) }
  end
end

local origin = vec(c.x, c.y, zt)
local function sky(az, el, r)          -- compass azimuth (north = +y, east = +x), elevation
  local a, e = math.rad(az), math.rad(el)
  return origin + vec(math.cos(e) * math.sin(a), math.cos(e) * math.cos(a), math.sin(e)) * r
end
emitter { name = "SAT", position = sky(45, 60, 2.5 * lambda), polarization = "rhcp", toward = origin }
emitter { name = "JAM", position = sky(jam_az, 20, 2 * lambda), polarization = vec(0.3, -0.5, 0.8) }

crpa { satellite = "SAT", elements = elements, jnr = 40, snr = -20, adapt = adapt, periods = 24,
       snapshot_periods = 24, log = "crpa.csv" }
view { steps_per_frame = 8 }
