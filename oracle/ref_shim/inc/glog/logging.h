// Forwards to the glog stand-in (reference-pin build only).
#pragma once
#include <ref_glog.hpp>
