/* Event.hpp -- TEST INFRASTRUCTURE ONLY: the event names and registration
 * calls used by src/Sim/BarnesHut.cpp (the UI's theta slider).  Registration
 * is a no-op here: the harness sets Octree::Theta directly. */
#pragma once
#include <functional>

enum class EEvent { BHThetaChanged };

struct EventData {
    virtual ~EventData() = default;
};
struct FloatEventData : public EventData {
    float Value;
    explicit FloatEventData(float v) : Value(v) {}
};

template <class T>
auto EventValue(const EventData& data) -> decltype(static_cast<const T&>(data).Value) {
    return static_cast<const T&>(data).Value;
}

class EventStream {
public:
    static void Register(EEvent, std::function<void(const EventData&)>) {}
    static void UnregisterAll(EEvent) {}
};
