// Forwards to the Boost.Serialization stand-in (reference-pin build only).
#pragma once
#include <ref_boost.hpp>
