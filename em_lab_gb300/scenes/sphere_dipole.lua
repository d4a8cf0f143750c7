-- 128^3 plain-method case: a point dipole at the centre beside a dielectric sphere.
-- Same scene as em_lab_gb300.configs.plain_small(), written with the scene API.
scene {
  name        = "Dipole beside a dielectric sphere",
  description = "Hertzian dipole, eps_r 2.25 sphere 30 cells to +x, 10-cell absorber.",
  size        = {128, 128, 128},
  wavelength  = 16,
  courant     = 0.5,
  pml         = 10,
}

local c = grid.center
sphere  { center = c + vec(30, 0, 0), radius = 10, material = { name = "sphere glass", epsilon_r = 2.25 } }
dipole  { center = c, orientation = "z", length = 0, amplitude = 7 }   -- ideal point current
probe   { position = c - vec(30, 0, 0), name = "behind" }
flux_box { min = {52, 52, 52}, max = {76, 76, 76}, name = "radiated" }
far_field {}
view { steps_per_frame = 2 }
