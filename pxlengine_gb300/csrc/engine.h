// Engine internals shared between the host translation units.
#pragma once

namespace pxf {

// Default P2G tile shape index (PXF_P2G_TILE environment variable, else 0).
int p2g_shape_index();
int p2g_lanes_default();

// PXF_TRACE=1: one line per library step on stderr (flushed), for locating host-side failures.
bool trace_on();
void trace(const char* fmt, ...);

}  // namespace pxf
