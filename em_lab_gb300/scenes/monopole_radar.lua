-- Pulsed radar: a 6 x 6 array of probe-fed square patches over a ground plate images a metal
-- sphere. The centre 2 x 2 patches transmit a Gaussian pulse and all 36 receive. The first pass runs
-- without the sphere (calibration), the second with it; the radar reports its detections.
local lambda = 20
local pml    = 10
scene { name = "Patch-array radar", size = {200, 128, 128}, pml = pml, wavelength = lambda }

local N, d    = 6, 12                   -- patches per side, spacing (cells)
local P, h    = 9, 2                    -- patch side, height over the ground plate (cells)
local inset   = 2                       -- probe distance from the patch edge (cells)
local xg      = pml + 6                 -- ground plate
local c       = grid.center
local dist = param { name = "range", label = "sphere distance (cells)", default = 90, min = 60, max = 140, step = 10 }
local side = param { name = "offset", label = "sphere offset along y (cells)", default = 10, min = -20, max = 20, step = 5 }

local half = (N - 1) * d / 2
sheet { min = vec(xg, c.y - half - P, c.z - half - P), max = vec(xg, c.y + half + P, c.z + half + P) }
for i = 0, N - 1 do
  for j = 0, N - 1 do
    local y0 = c.y - half + i * d - math.floor(P / 2)
    local z0 = c.z - half + j * d - math.floor(P / 2)
    sheet { min = vec(xg + h, y0, z0), max = vec(xg + h, y0 + P, z0 + P) }
    local transmits = (i == 2 or i == 3) and (j == 2 or j == 3)
    monopole {
      base = vec(xg, y0 + inset, z0 + math.floor(P / 2)), orientation = "+x", length = h, waveform = "pulse",
      pulse_width = 0.5, amplitude = transmits and 1 or 0, name = string.format("p[%d,%d]", i + 1, j + 1),
    }
  end
end

sphere { center = vec(xg + h + dist, c.y + side, c.z), radius = 12, material = "metal", target = true, name = "sphere" }
radar { range = {20, 150}, fov = 25, phase_center = vec(1.5, math.floor(P / 2) - inset, 0), log = "radar.csv" }
view { steps_per_frame = 8 }
