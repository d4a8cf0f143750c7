-- A plane wave through two slits in a metal wall; power through a plane behind the wall.
scene { name = "Two slits", size = {128, 96, 64}, wavelength = 16, pml = 10 }

local gap = param { name = "spacing", label = "slit spacing (cells)", default = 24, min = 8, max = 48, step = 4 }

wall { axis = "x", position = 48, thickness = 2, slits = { count = 2, width = 6, spacing = gap, direction = "z" } }
plane_wave { axis = "x", position = 20, polarization = "z", amplitude = 1 }
probe { position = {90, 48, 32}, name = "screen" }
flux_plane { axis = "x", position = 100, name = "transmitted" }
for i, y in ipairs({36, 60}) do
  probe { position = {60, y, 32}, name = string.format("slit%d", i) }
end
