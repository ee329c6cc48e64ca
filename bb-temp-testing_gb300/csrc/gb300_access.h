// Library-internal access to the device handles behind the C++ classes, for
// the canvas-to-optimiser hand-off (gb300_ext.h). Each member is defined in
// the translation unit that owns the class's Device struct.
#pragma once

#include "vm_capi.h"

namespace voromesh {

class VoroOptimizer;
class Canvas;

struct Gb300Access {
    static vm_optimizer *handle(VoroOptimizer &opt); // voro_optimizer.cpp
    static cv_canvas *handle(const Canvas &canvas);  // canvas.cpp
    static void refresh(VoroOptimizer &opt);         // voro_optimizer.cpp: re-read the host-side counters
};

} // namespace voromesh
