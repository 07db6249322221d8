// Internal constants of the device labeller (sf_label.cu).
#pragma once

namespace sf {

// Frames labelled together in one batch.
constexpr int kLabelMaxBatch = 64;

} // namespace sf
