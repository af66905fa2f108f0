/* Build shim for the vendored IlmBase exception sources, whose pre-generated
   configuration header declares a Windows platform: the only Windows call
   they make is a debugger trap behind an environment variable. */
#pragma once
static inline void DebugBreak(void) {}
