// bicos_gb300 C++ entry point: libBICOS include/match.hpp:31-41.
#pragma once

#include "common.hpp"

namespace BICOS {

// Matches two stacks of n rectified device images (IMG_8U or IMG_16U, one
// size).  `disparity` is (re)created as IMG_16S, or IMG_32F when a subpixel
// step is set; `corrmap`, when given and a threshold is set, as IMG_32F or
// IMG_64F by precision.  Work is enqueued on `stream` and this returns
// without waiting for it.  Throws BICOS::Exception, or std::invalid_argument
// for stacks whose descriptor would exceed 256 bits, as the reference does.
void match(const std::vector<Image>& stack0, const std::vector<Image>& stack1, Image& disparity,
           Config cfg = Config {}, Image* corrmap = nullptr, Stream stream = nullptr);

}  // namespace BICOS
