/* Stub for building the reference's BLAZE_gpu sources as the oracle's
 * cross-check (test infrastructure only). BLAZE_gpu/util.hpp includes this
 * boost header but uses only std::hash, so nothing from boost is needed. */
#pragma once
