-- Half-wave thin-wire dipole with a 50-ohm resistive feed, swept with a Gaussian pulse.
scene { name = "Fed thin-wire dipole", size = {96, 96, 112}, wavelength = 32, pml = 12 }

local length = param { name = "length", label = "length (cells)", default = 15, min = 7, max = 31, step = 2 }
local radius = param { name = "radius", label = "wire radius (cells)", default = 0.08, min = 0.01, max = 0.3, step = 0.01 }

dipole {
  center = grid.center, orientation = "z", length = length, radius = radius,
  waveform = "pulse", pulse_width = 0.4, impedance = 50, name = "feed",
}
sweep { wavelengths = {20, 60}, points = 64 }
probe { position = grid.center + vec(20, 0, 0), name = "near" }
far_field { margin = 3 }
