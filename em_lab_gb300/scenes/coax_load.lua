-- A 50-ohm square coaxial line of voxels, driven at one end and terminated at the other.
scene { name = "Coax line", size = {160, 40, 40}, wavelength = 32, pml = 8 }

local term = param { name = "termination", label = "far end", choices = {"load", "open", "short"} }
local cable = coax { from = vec(20, 20, 20), axis = "+x", length = 120, z0 = 50, termination = term }
print(string.format("coax: Z0 %.2f ohm, eps_r %.3f, line wavelength %.2f cells", cable.z0, cable.epsilon_r,
                    cable.wavelength))
view { steps_per_frame = 8 }
