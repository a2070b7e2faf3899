// The render context behind integration/render_gpu.cpp, for code that reads the
// last frame straight from the device (integration/output_gpu.cpp).
#pragma once

#include "forkerrenderer.h"

// The context Render::Preconfigure created (NULL before it).
fr_ctx* RenderGpuContext();
