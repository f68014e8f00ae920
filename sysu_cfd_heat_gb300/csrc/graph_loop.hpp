// Device-side control flow for the iterative solves: CUDA graph conditional
// nodes (a WHILE loop whose body's last kernel decides whether it runs again,
// an IF whose condition an earlier kernel sets).  A solve whose loop lives in
// the graph never waits for the host, so it can sit inside a larger captured
// graph (the case batch) and, run alone, costs no host round trip per chunk of
// iterations.
//
// The helpers append to the capture in progress on a stream: the node joins
// the stream's current dependencies and becomes the stream's new dependency;
// its body is captured from a second stream into the node's body graph.
#pragma once

#include <cuda_runtime.h>

#include <functional>

namespace sysu {

// True when work enqueued on st is being captured into a graph.
bool stream_capturing(cudaStream_t st);

// A conditional handle of the graph being captured on st, with the given
// value applied at every launch of that graph.
cudaGraphConditionalHandle graph_cond_handle(cudaStream_t st, unsigned default_value);

// Appends a conditional node (cudaGraphCondTypeWhile or cudaGraphCondTypeIf)
// with handle h to the capture in progress on st; body(side) enqueues the
// node's body on `side`, a stream that is not capturing.
void graph_cond_node(cudaStream_t st, cudaStream_t side, cudaGraphConditionalHandle h,
                     cudaGraphConditionalNodeType type, const std::function<void(cudaStream_t)> &body);

// The last kernel of a WHILE body: *count += 1 and the loop goes on while
// *stop is 0 and *count < bound.  bound keeps every loop finite.
void graph_loop_tail(cudaGraphConditionalHandle h, const int *stop, int *count, int bound, cudaStream_t st);

// Sets an IF node's condition to (*flag != 0).
void graph_if_flag(cudaGraphConditionalHandle h, const int *flag, cudaStream_t st);

// A stream that is never captured, for building node bodies (one per thread
// and device, created on first use).
cudaStream_t graph_side_stream();

// Self-test of the loop's two exits: a WHILE node whose body counts its runs and
// sets the stop flag after `stop_at` of them (never, for stop_at <= 0), with the
// given bound; returns the number of bodies that ran (min(stop_at, bound)).
int graph_loop_selftest(int bound, int stop_at, cudaStream_t st);

}  // namespace sysu
