// Shim of thrust's static-assert header for the host lane emulator — TEST
// INFRASTRUCTURE ONLY.  The reference uses just this one macro from thrust.
#pragma once
#define THRUST_STATIC_ASSERT(x) static_assert(x, #x)
