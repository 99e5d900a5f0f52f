// lt_order.h -- ordering of a context's GPU work across stream switches and of
// the host writes into buffers that queued GPU work still reads.
//
// Two rules, kept in one place so that they can be checked without a GPU
// (tests/native/order_check.cpp runs them over a recording runtime):
//
// 1. Stream switch. lt_set_stream moves a context from stream A to stream B.
//    Work already queued on A (a batched differentiable render returns once
//    queued; device-buffer lt_intersect too) must finish before anything the
//    context queues on B touches the same buffers, so the switch records an
//    event on A and makes B wait for it. The host does not block.
//
// 2. Host rewrite of a buffer read by queued work. The batched renders upload
//    the scene table from one pinned host copy into one device copy. After
//    queuing a reader of the table (the captured batch loop, a batched
//    differentiable kernel), the context records a "table free" event on its
//    stream; before the host writes the pinned copy again it waits for that
//    event. The device copy needs no host wait: the next upload is queued on
//    the context's stream, which (rule 1) is ordered after every earlier reader.
//
// Rt is the runtime: the real one wraps cudaEventRecord / cudaStreamWaitEvent /
// cudaEventSynchronize; the test's records the calls.
#pragma once

namespace lt {

template <class Rt>
struct WorkOrder {
    typename Rt::Event switch_ev{};  // recorded on the old stream at a switch
    typename Rt::Event table_ev{};   // recorded after the last queued table reader
    bool table_pending = false;      // a reader was queued since the last host wait

    // Rule 1. Returns the runtime's status (0 = success).
    int switch_stream(Rt &rt, typename Rt::Stream from, typename Rt::Stream to) {
        if (from == to) return 0;
        int e = rt.record(switch_ev, from);
        if (e == 0) e = rt.wait(to, switch_ev);
        return e;
    }

    // Rule 2, after queuing a reader of the table on `stream`.
    int table_read_queued(Rt &rt, typename Rt::Stream stream) {
        const int e = rt.record(table_ev, stream);
        if (e == 0) table_pending = true;
        return e;
    }

    // Rule 2, before the host writes the pinned table.
    int before_table_write(Rt &rt) {
        if (!table_pending) return 0;
        const int e = rt.sync(table_ev);
        if (e == 0) table_pending = false;
        return e;
    }
};

}  // namespace lt
