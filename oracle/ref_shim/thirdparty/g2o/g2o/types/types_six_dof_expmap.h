// Forwards to the g2o stand-in (reference-pin build only).
#pragma once
#include <ref_g2o.hpp>
