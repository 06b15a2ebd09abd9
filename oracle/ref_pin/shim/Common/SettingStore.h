// Stand-in for glim::SettingStore / TimeStat (UI-only; never executed by the pin driver).
#pragma once
namespace glim {
struct SettingStore {
    template <typename T> bool Combo(const char*, T*) { return false; }
    template <typename T, typename S> bool Slider(const char*, T*, S, T, T) { return false; }
    bool Checkbox(const char*, bool*) { return false; }
};
struct TimeStat {
    void Begin() {}
    void End() {}
    void AddSample(double) {}
    void Draw(const char*) {}
    void GetElapsedMs(double& mean, double& dev) const { mean = 1.0; dev = 0.0; }
};
}  // namespace glim
