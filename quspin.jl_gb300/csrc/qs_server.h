// qs_server.h -- the request loop behind qs_server_* (qs_server.cpp).
#pragma once

#include "../../include/qsgpu.h"

namespace qs {

struct Server;
Server* server_create(const qs_server_opts* opts);
void server_destroy(Server* s);
int64_t server_submit(Server* s, const qs_request* r);
int server_poll(Server* s, int64_t ticket, qs_result* out);
int server_wait(Server* s, int64_t ticket, double timeout_s, qs_result* out);
void server_vector(Server* s, int64_t ticket, double* out, int64_t len);
void server_release(Server* s, int64_t ticket);
void server_stats(Server* s, qs_server_counters* out);

}  // namespace qs
