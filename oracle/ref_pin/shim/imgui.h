// Stand-in for the few ImGui calls in the reference renderer (never executed by the pin driver).
#pragma once
enum ImGuiKey { ImGuiKey_F9 = 0 };
namespace ImGui {
inline void SeparatorText(const char*) {}
inline void PushItemWidth(float) {}
inline void PopItemWidth() {}
inline void Separator() {}
inline void Text(const char*, ...) {}
inline bool IsKeyPressed(ImGuiKey) { return false; }
}  // namespace ImGui
