// pk_events.h — host-side dispatch of the step's collision begin/end events to waiters, the part of
// the reference's task handler that consumes them (task_handler::on_collision / on_collision_exit /
// on_destruction, core/co.h:495-595; awaitables wait_for_collision / wait_for_separation /
// wait_until_destroyed, core/awaitables.h:136-252, 260-300). Plain C++ (no CUDA), so the matching
// rules are tested on the CPU.
//
// Rules, as in the reference:
//  - a waiter watches one object, for a begin (collision) or end (separation) event, either with a
//    given other object or with any (`with` = kAny);
//  - an event (a, b) is offered to a's waiters, then to b's; every matching waiter of that object
//    fires on it (in registration order) and is removed;
//  - destroying an object fails its collision and separation waiters and the waiters elsewhere that
//    name it as `with` (error "object destroyed"), and fires its destruction waiters.
#pragma once

#include <cstdint>
#include <unordered_map>
#include <vector>

namespace pk
{

struct Wake
{
    uint64_t waiter;
    uint64_t object;
    uint64_t other; // the colliding / separating object; kAny for destruction and failures
    int32_t kind;   // 1 collision, 2 separation, 3 destroyed
    int32_t failed; // 1: the waiter ended because an object it needed was destroyed
};

class EventDispatcher
{
public:
    static constexpr uint64_t kAny = ~uint64_t(0);
    enum : int32_t
    {
        COLLISION = 1,
        SEPARATION = 2,
        DESTROYED = 3
    };

    uint64_t add(int32_t kind, uint64_t object, uint64_t with)
    {
        const uint64_t id = next_++;
        by_object_[object].push_back({id, kind, object, kind == DESTROYED ? kAny : with});
        return id;
    }

    bool cancel(uint64_t id)
    {
        for (auto &kv : by_object_)
            for (size_t i = 0; i < kv.second.size(); ++i)
                if (kv.second[i].id == id)
                {
                    kv.second.erase(kv.second.begin() + long(i));
                    return true;
                }
        return false;
    }

    size_t pending() const
    {
        size_t n = 0;
        for (const auto &kv : by_object_) n += kv.second.size();
        return n;
    }

    // One begin (kind 1) or end (kind 2) event between objects a and b.
    void event(int32_t kind, uint64_t a, uint64_t b, std::vector<Wake> &out)
    {
        offer(kind, a, b, out);
        offer(kind, b, a, out);
    }

    // Object removed from the world.
    void destroyed(uint64_t obj, std::vector<Wake> &out)
    {
        auto it = by_object_.find(obj);
        if (it != by_object_.end())
        {
            for (const W &w : it->second)
                out.push_back({w.id, obj, kAny, w.kind, w.kind == DESTROYED ? 0 : 1});
            by_object_.erase(it);
        }
        for (auto &kv : by_object_)
        {
            auto &v = kv.second;
            for (size_t i = 0; i < v.size();)
            {
                if (v[i].kind != DESTROYED && v[i].with == obj)
                {
                    out.push_back({v[i].id, v[i].object, kAny, v[i].kind, 1});
                    v.erase(v.begin() + long(i));
                }
                else
                    ++i;
            }
        }
    }

private:
    struct W
    {
        uint64_t id;
        int32_t kind;
        uint64_t object, with;
    };

    void offer(int32_t kind, uint64_t obj, uint64_t other, std::vector<Wake> &out)
    {
        auto it = by_object_.find(obj);
        if (it == by_object_.end()) return;
        auto &v = it->second;
        for (size_t i = 0; i < v.size();)
        {
            if (v[i].kind == kind && (v[i].with == kAny || v[i].with == other))
            {
                out.push_back({v[i].id, obj, other, kind, 0});
                v.erase(v.begin() + long(i));
            }
            else
                ++i;
        }
        if (v.empty()) by_object_.erase(it);
    }

    std::unordered_map<uint64_t, std::vector<W>> by_object_;
    uint64_t next_ = 1;
};

} // namespace pk
