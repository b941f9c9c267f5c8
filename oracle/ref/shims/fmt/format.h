// Declarations that let Core/RenderSetting.h specialise fmt::formatter.
// The specialisation's body is a template that the oracle build never instantiates.
#pragma once
namespace fmt {
template <typename T, typename Char = char, typename Enable = void>
struct formatter;
}
