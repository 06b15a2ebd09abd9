// Stand-in for the reference's OpenGL wrapper: types and constants only, so that
// the renderer parts of the compiled files build.  Nothing here touches a GPU.
#pragma once
#include <cstddef>
#include <cstdint>
#include <memory>
#include <string_view>
using GLuint = uint32_t;
using GLint64 = int64_t;
using GLbitfield = uint32_t;
enum : uint32_t {
    GL_RGBA8 = 1, GL_RGBA16F, GL_R32F, GL_RG16F, GL_R8UI, GL_RG8UI, GL_DYNAMIC_STORAGE_BIT, GL_MAP_WRITE_BIT,
    GL_MAP_READ_BIT, GL_MAP_PERSISTENT_BIT, GL_MAP_FLUSH_EXPLICIT_BIT, GL_TIME_ELAPSED, GL_QUERY_RESULT,
    GL_TEXTURE_CUBE_MAP_SEAMLESS
};
namespace ogl {
struct Texture2D {
    uint32_t Width = 0, Height = 0;
    Texture2D(uint32_t w, uint32_t h, uint32_t, uint32_t) : Width(w), Height(h) {}
};
struct TextureCube {};
struct Buffer {
    size_t Size = 0;
    std::unique_ptr<uint8_t[]> Host;
    Buffer(size_t size, GLbitfield, const void* = nullptr) : Size(size), Host(new uint8_t[size]()) {}
    template <typename T>
    struct Mapping {
        T* p;
        T* operator->() const { return p; }
        T& operator*() const { return *p; }
        void reset() {}
        T* release() { return p; }
    };
    template <typename T>
    Mapping<T> Map(GLbitfield) { return Mapping<T>{reinterpret_cast<T*>(Host.get())}; }
    void FlushMappedRange(size_t, size_t) {}
};
struct Shader {
    template <typename T>
    void SetUniform(std::string_view, const T&) {}
    void DispatchCompute(uint32_t, uint32_t, uint32_t) {}
    void DispatchFullscreen() {}
};
}  // namespace ogl
