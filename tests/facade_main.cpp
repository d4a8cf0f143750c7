// Drives the C++ SimulationGrid facade the way the reference's Application does
// (configure -> uploadMaterials -> setSources -> step), printing a field checksum.
#include <cmath>
#include <cstdio>

#include "emlab_simulation_grid.hpp"

int main() {
    using namespace emlab_cpp;
    try {
        SimulationGrid grid;
        GridConfig cfg;
        cfg.size = {40, 36, 32};
        cfg.pmlThickness = 6;
        grid.configure(cfg);
        MaterialVolume m(grid.size());
        for (int z = 10; z < 14; ++z)
            for (int y = 10; y < 14; ++y)
                for (int x = 10; x < 14; ++x) m.set({x, y, z}, 0.02f, 2.5f);
        grid.uploadMaterials(m);
        emlab_source s{};
        s.center[0] = 20, s.center[1] = 18, s.center[2] = 16;
        s.softness[0] = s.softness[1] = s.softness[2] = 0.75f;
        s.polarization[2] = 1.0f;
        s.amplitude = 3.0f, s.wavelength = 12.0f, s.ramp_periods = 1.0f, s.enabled = 1;
        grid.setSources({s});
        int callbacks = 0;
        grid.step(10, [&] { ++callbacks; });
        grid.step(30);
        grid.synchronize();
        // device view of the state (eFieldTexture / bFieldTexture): non-null arrays, row pitch >= nx
        const SimulationGrid::FieldView view = grid.fieldView();
        bool view_ok = view.pitch >= grid.size().x && view.plane >= (long long)view.pitch * grid.size().y;
        for (float* p : view.component) view_ok = view_ok && p != nullptr;
        MaterialVolume wrong({8, 8, 8});
        bool threw = false;
        try {
            grid.uploadMaterials(wrong);
        } catch (const std::runtime_error&) {
            threw = true;
        }
        std::printf("steps %llu time %.3f callbacks %d size-mismatch-throws %d field-view %d\n",
                    (unsigned long long)grid.stepCount(), grid.time(), callbacks, threw ? 1 : 0, view_ok ? 1 : 0);
        return (grid.stepCount() == 40 && callbacks == 10 && threw && view_ok) ? 0 : 1;
    } catch (const std::runtime_error& e) {
        std::printf("runtime_error: %s\n", e.what());
        return 3;
    }
}
