// Host check of physkit_gb300/csrc/pk_events.h (compiled with g++): the waiter rules of the
// reference's task handler (core/co.h:495-595, core/awaitables.h:136-300).
#include "../../physkit_gb300/csrc/pk_events.h"

#include <cstdio>
#include <vector>

using namespace pk;

static int fails = 0;
#define CHECK(c)                                                                                   \
    do                                                                                             \
    {                                                                                              \
        if (!(c))                                                                                  \
        {                                                                                          \
            std::printf("check failed line %d: %s\n", __LINE__, #c);                              \
            ++fails;                                                                               \
        }                                                                                          \
    } while (0)

int main()
{
    const uint64_t A = 10, B = 11, C = 12, ANY = EventDispatcher::kAny;
    {
        // with-filter, any, and both sides: a's waiters first, then b's
        EventDispatcher d;
        std::vector<Wake> out;
        uint64_t w1 = d.add(1, A, B);   // A with B
        uint64_t w2 = d.add(1, A, C);   // A with C: not this event
        uint64_t w3 = d.add(1, B, ANY); // B with anything
        uint64_t w4 = d.add(2, A, ANY); // separation: not a begin event
        d.event(1, A, B, out);
        CHECK(out.size() == 2);
        CHECK(out[0].waiter == w1 && out[0].object == A && out[0].other == B && out[0].kind == 1 && !out[0].failed);
        CHECK(out[1].waiter == w3 && out[1].object == B && out[1].other == A);
        CHECK(d.pending() == 2);
        out.clear();
        d.event(2, B, A, out); // separation, objects in the other order
        CHECK(out.size() == 1 && out[0].waiter == w4 && out[0].object == A && out[0].other == B);
        out.clear();
        d.event(1, C, A, out);
        CHECK(out.size() == 1 && out[0].waiter == w2 && out[0].other == C);
        CHECK(d.pending() == 0);
    }
    {
        // every matching waiter of an object fires on one event, in registration order; fired once
        EventDispatcher d;
        std::vector<Wake> out;
        uint64_t w1 = d.add(1, A, ANY), w2 = d.add(1, A, B), w3 = d.add(1, A, ANY);
        d.event(1, B, A, out);
        CHECK(out.size() == 3 && out[0].waiter == w1 && out[1].waiter == w2 && out[2].waiter == w3);
        out.clear();
        d.event(1, B, A, out);
        CHECK(out.empty());
    }
    {
        // destruction: the object's collision/separation waiters fail, its destruction waiters fire,
        // waiters on other objects that name it fail; cancel removes a waiter
        EventDispatcher d;
        std::vector<Wake> out;
        uint64_t w1 = d.add(1, A, ANY), w2 = d.add(3, A, ANY), w3 = d.add(2, B, A), w4 = d.add(1, B, C);
        uint64_t w5 = d.add(1, C, ANY);
        CHECK(d.cancel(w5) && !d.cancel(w5));
        d.destroyed(A, out);
        CHECK(out.size() == 3);
        bool s1 = false, s2 = false, s3 = false;
        for (const Wake &k : out)
        {
            if (k.waiter == w1) s1 = k.failed == 1 && k.kind == 1;
            if (k.waiter == w2) s2 = k.failed == 0 && k.kind == 3;
            if (k.waiter == w3) s3 = k.failed == 1 && k.object == B;
        }
        CHECK(s1 && s2 && s3);
        CHECK(d.pending() == 1); // w4 stays
        out.clear();
        d.event(1, B, C, out);
        CHECK(out.size() == 1 && out[0].waiter == w4);
    }
    std::printf("event_check_failures=%d\n", fails);
    return fails ? 1 : 0;
}
