// order_check.cpp -- the context's work-ordering rules (lantern_gb300/csrc/lt_order.h)
// over a runtime that records its calls instead of reaching CUDA. Prints "ok"
// and exits 0 when every check holds; otherwise names the failed check.
#include <stdio.h>

#include <string>
#include <vector>

#include "lt_order.h"

namespace {

struct RecordingRt {
    using Event = int;
    using Stream = int;
    std::vector<std::string> log;
    int fail_next = 0;  // nonzero: the next call returns this status
    int status() {
        const int e = fail_next;
        fail_next = 0;
        return e;
    }
    int record(Event e, Stream s) {
        log.push_back("record ev" + std::to_string(e) + " on s" + std::to_string(s));
        return status();
    }
    int wait(Stream s, Event e) {
        log.push_back("s" + std::to_string(s) + " waits ev" + std::to_string(e));
        return status();
    }
    int sync(Event e) {
        log.push_back("host waits ev" + std::to_string(e));
        return status();
    }
};

int failures = 0;

void expect(bool ok, const char *what) {
    if (!ok) {
        fprintf(stderr, "FAILED: %s\n", what);
        ++failures;
    }
}

bool log_is(const RecordingRt &rt, const std::vector<std::string> &want) { return rt.log == want; }

}  // namespace

int main() {
    using Order = lt::WorkOrder<RecordingRt>;
    {  // a switch to another stream: the new stream waits for the old one's work
        RecordingRt rt;
        Order o;
        o.switch_ev = 7;
        expect(o.switch_stream(rt, 1, 2) == 0, "switch returns success");
        expect(log_is(rt, {"record ev7 on s1", "s2 waits ev7"}), "switch records on the old stream, new one waits");
    }
    {  // setting the same stream again orders nothing
        RecordingRt rt;
        Order o;
        expect(o.switch_stream(rt, 3, 3) == 0 && rt.log.empty(), "same stream: no event");
    }
    {  // a table rewrite with no reader queued does not block the host
        RecordingRt rt;
        Order o;
        o.table_ev = 5;
        expect(o.before_table_write(rt) == 0 && rt.log.empty(), "first table write: no wait");
    }
    {  // a reader queued on stream A, then a switch to B, then a rewrite:
       // the host waits for A's reader before touching the pinned table
        RecordingRt rt;
        Order o;
        o.switch_ev = 1;
        o.table_ev = 2;
        expect(o.table_read_queued(rt, 10) == 0, "reader recorded");
        expect(o.switch_stream(rt, 10, 20) == 0, "switch");
        expect(o.before_table_write(rt) == 0, "rewrite");
        expect(log_is(rt, {"record ev2 on s10", "record ev1 on s10", "s20 waits ev1", "host waits ev2"}),
               "rewrite waits on the previous reader's event");
        // the wait is spent: a second rewrite without a new reader does not wait again
        rt.log.clear();
        expect(o.before_table_write(rt) == 0 && rt.log.empty(), "second rewrite: no wait");
    }
    {  // every reader re-arms the wait, on the stream it was queued on
        RecordingRt rt;
        Order o;
        o.table_ev = 4;
        o.table_read_queued(rt, 1);
        o.before_table_write(rt);
        o.table_read_queued(rt, 9);
        o.before_table_write(rt);
        expect(log_is(rt, {"record ev4 on s1", "host waits ev4", "record ev4 on s9", "host waits ev4"}),
               "each reader re-arms the wait");
    }
    {  // a failed host wait keeps the wait armed (the next rewrite waits again)
        RecordingRt rt;
        Order o;
        o.table_ev = 3;
        o.table_read_queued(rt, 1);
        rt.fail_next = 700;
        expect(o.before_table_write(rt) == 700, "failed wait returns the runtime's status");
        expect(o.table_pending, "failed wait stays armed");
        expect(o.before_table_write(rt) == 0 && !o.table_pending, "retry waits and disarms");
    }
    {  // a failed record at a switch is reported and the new stream is not made to wait on it
        RecordingRt rt;
        Order o;
        rt.fail_next = 1;
        expect(o.switch_stream(rt, 1, 2) == 1, "failed record returns its status");
        expect(rt.log.size() == 1, "no wait after a failed record");
    }
    if (failures) return 1;
    printf("ok\n");
    return 0;
}
