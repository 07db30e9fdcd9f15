// Forwards to the OpenCV stand-in (reference-pin build only).
#pragma once
#include <ref_cv.hpp>
