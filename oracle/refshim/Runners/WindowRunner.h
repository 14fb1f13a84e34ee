// Test infrastructure only (oracle build of the reference). Header-only
// stand-in for the reference's Runners/WindowRunner.h, which pulls in the
// OpenGL text renderer. Camera::update (Raytracing/Camera.cpp:48-284) only
// polls the window for input; the oracle harness answers "no input", so the
// non-interactive camera path runs unchanged. Key codes are arbitrary
// distinct values (no input is ever reported for any of them).
#pragma once
#include <cstdint>

namespace Raycer
{
    enum ShimKeyCodes
    {
        GLFW_KEY_A = 1, GLFW_KEY_D, GLFW_KEY_DELETE, GLFW_KEY_DOWN, GLFW_KEY_E, GLFW_KEY_HOME,
        GLFW_KEY_INSERT, GLFW_KEY_LEFT, GLFW_KEY_LEFT_ALT, GLFW_KEY_LEFT_CONTROL, GLFW_KEY_LEFT_SHIFT,
        GLFW_KEY_PAGE_DOWN, GLFW_KEY_PAGE_UP, GLFW_KEY_Q, GLFW_KEY_RIGHT, GLFW_KEY_RIGHT_ALT,
        GLFW_KEY_RIGHT_CONTROL, GLFW_KEY_RIGHT_SHIFT, GLFW_KEY_S, GLFW_KEY_SPACE, GLFW_KEY_UP, GLFW_KEY_W,
        GLFW_MOUSE_BUTTON_LEFT, GLFW_MOUSE_BUTTON_MIDDLE, GLFW_MOUSE_BUTTON_RIGHT
    };

    struct MouseInfo
    {
        int64_t windowX = 0;
        int64_t windowY = 0;
        int64_t scaledX = 0;
        int64_t scaledY = 0;
        int64_t deltaX = 0;
        int64_t deltaY = 0;
        double scrollY = 0.0;
        bool hasScrolled = false;
    };

    class WindowRunner
    {
    public:
        const MouseInfo& getMouseInfo() const { return mouseInfo; }
        bool keyIsDown(int32_t) { return false; }
        bool mouseIsDown(int32_t) { return false; }
        bool keyWasPressed(int32_t) { return false; }
        bool mouseWasPressed(int32_t) { return false; }
        double getMouseWheelScroll() { return 0.0; }
        double getElapsedTime() const { return 0.0; }
    private:
        MouseInfo mouseInfo;
    };
}
