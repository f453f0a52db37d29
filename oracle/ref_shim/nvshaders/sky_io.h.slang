// Stand-in for nvpro_core2's nvshaders/sky_io.h.slang, which the reference's
// shaders/shaderio.h:26 includes and which is not part of the reference
// checkout. FrameConstants ends with its SkySimpleParameters (shaderio.h:260);
// the sky is not on the tessellation path, so the layout pins stop before that
// field and this opaque placeholder only lets the header compile.
// TEST INFRASTRUCTURE (oracle side).
#pragma once
struct SkySimpleParameters
{
  float opaque[4];
};
