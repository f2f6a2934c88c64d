// Shims that let the reference NSL headers compile in this image without their absent dependencies (no reference
// file is edited). TEST INFRASTRUCTURE ONLY. Include before any NSL header.
//   * NSL::Logger (spdlog + CLI11, src/NSL/logger.hpp): fmt-based, records the last message;
//   * the Generic lattice (yaml-cpp, src/NSL/Lattice/Implementations/generic.hpp): excluded by its include guard;
//   * torch::linalg::eigh(t, uplo) (src/NSL/LinAlg/eigh.tpp:13): mapped onto at::linalg_eigh.
#pragma once
#include <fmt/format.h>
#include <torch/torch.h>

#include <string>

#define NSL_LOGGER_INCLUDE_HPP
#define NSL_LATTICE_GENERIC_HPP
#define NSL_LATTICE_GENERIC_TPP

namespace NSL::Logger {
inline std::string last_message;
inline bool do_profile = false;
template <class... A> void info(fmt::format_string<A...> f, A &&...a) { last_message = fmt::format(f, std::forward<A>(a)...); }
template <class... A> void debug(fmt::format_string<A...>, A &&...) {}
template <class... A> void warn(fmt::format_string<A...> f, A &&...a) { last_message = fmt::format(f, std::forward<A>(a)...); }
template <class... A> void error(fmt::format_string<A...> f, A &&...a) { last_message = fmt::format(f, std::forward<A>(a)...); }
}  // namespace NSL::Logger

namespace torch::linalg {
inline std::tuple<at::Tensor, at::Tensor> eigh(const at::Tensor &t, std::string uplo) { return at::linalg_eigh(t, uplo); }
}  // namespace torch::linalg
