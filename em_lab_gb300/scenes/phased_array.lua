-- Planar phased array: N x N thin-wire dipoles (0.46 lambda, along x) at half-wavelength pitch,
-- a quarter wavelength over a ground sheet, under a 6-cell radome slab (eps_r 3.5). Every dipole
-- has a 50-ohm feed driven by a Gaussian pulse with a separable Taylor amplitude taper (nbar 4,
-- -30 dB sidelobes) and a true time delay that steers the beam to (theta, phi).
local lambda = 24
local pml    = 12
local N     = param { name = "elements", label = "elements per side", default = 16, min = 2, max = 16, step = 2 }
local theta = param { name = "theta", label = "steering theta (deg)", default = 20, min = 0, max = 60, step = 1 }
local phi   = param { name = "phi", label = "steering phi (deg)", default = 30, min = 0, max = 359, step = 1 }
local nxy   = param { name = "nxy", label = "grid x / y (cells)", default = 384, min = 96, max = 512, step = 32 }
local nz    = param { name = "nz", label = "grid z (cells)", default = 256, min = 96, max = 512, step = 32 }

scene { name = "Planar phased array", size = {nxy, nxy, nz}, pml = pml, wavelength = lambda }
material { name = "radome", epsilon_r = 3.5 }

local c     = grid.center
local pitch = lambda / 2
local inner = pml + 20                  -- the far-field box lies this far in (everything radiating is inside)
local zg    = inner + 4                 -- ground sheet
local zd    = zg + lambda / 4           -- dipole plane
local zr    = zd + lambda               -- radome slab
local span  = (N - 1) * pitch / 2 + pitch

sheet { min = vec(c.x - span, c.y - span, zg), max = vec(c.x + span, c.y + span, zg) }
box { min = vec(inner + 4, inner + 4, zr), max = vec(nxy - inner - 4, nxy - inner - 4, zr + 6), material = "radome" }

-- Taylor line-source weights at the element positions (Taylor 1955; nbar terms, sidelobe level sll dB)
local function taylor(n, nbar, sll)
  local A = math.log(10 ^ (-sll / 20) + math.sqrt(10 ^ (-sll / 10) - 1)) / math.pi
  local s2 = nbar * nbar / (A * A + (nbar - 0.5) ^ 2)
  local function fact(k) local f = 1 for i = 2, k do f = f * i end return f end
  local F = {}
  for m = 1, nbar - 1 do
    local p = 1
    for q = 1, nbar - 1 do p = p * (1 - m * m / (s2 * (A * A + (q - 0.5) ^ 2))) end
    F[m] = fact(nbar - 1) ^ 2 / (fact(nbar - 1 + m) * fact(nbar - 1 - m)) * p
  end
  local w, wmax = {}, 0
  for i = 1, n do
    local x = (i - 0.5) / n - 0.5          -- position over the aperture, -1/2 .. 1/2
    local v = 1
    for m = 1, nbar - 1 do v = v + 2 * F[m] * math.cos(2 * math.pi * m * x) end
    w[i] = v
    wmax = math.max(wmax, v)
  end
  for i = 1, n do w[i] = w[i] / wmax end
  return w
end
local taper = taylor(N, 4, -30)

-- True-time-delay steering: an element farther along the beam direction fires later.
local st, sp = math.sin(math.rad(theta)), math.rad(phi)
local ux, uy = st * math.cos(sp), st * math.sin(sp)
local delays, dmin = {}, math.huge
for i = 1, N do
  for j = 1, N do
    local x, y = (i - 1 - (N - 1) / 2) * pitch, (j - 1 - (N - 1) / 2) * pitch
    local d = (x * ux + y * uy) / lambda    -- periods (c = 1 cell per unit time, period = lambda)
    delays[(i - 1) * N + j] = d
    dmin = math.min(dmin, d)
  end
end
for i = 1, N do
  for j = 1, N do
    local x, y = c.x + (i - 1 - (N - 1) / 2) * pitch, c.y + (j - 1 - (N - 1) / 2) * pitch
    dipole { center = vec(x, y, zd), orientation = "x", length = 11, radius = 0.05, impedance = 50,
             amplitude = taper[i] * taper[j], waveform = "pulse", pulse_width = 0.4,
             delay = 1 + delays[(i - 1) * N + j] - dmin, name = string.format("d[%d,%d]", i, j) }
  end
end
