"""Client side of the served form: drives an rt_server with a timed request
stream (``scenes.served_requests``) and collects results on a second thread.

The client keeps a mirror of the server's recency order (every add_scene and
submit advances it by one, as the server's submission clock does) so that it
never targets a scene that an upload has displaced under the scene cap.  An
upload's scene id is known at submit (rt_server_upload) and is a render
target from then on; the server holds such renders until the build is done.
The sequence of scenes, cameras, sizes and depths is therefore the same for
every server configuration, and images can be compared request by request."""
import queue
import threading
import time
import zlib

import numpy as np

from . import capi


class SceneCache:
    """Host copies of the workload's scenes, made once."""

    def __init__(self, wl):
        self.wl = wl
        self._made = {}

    def get(self, spec):
        if spec not in self._made:
            self._made[spec] = self.wl["make"](spec)
        return self._made[spec]


def _pace(t0, t):
    """Sleeps until t0 + t (perf_counter seconds), spinning the last 0.2 ms."""
    while True:
        d = t0 + t - time.perf_counter()
        if d <= 0:
            return
        if d > 2e-4:
            time.sleep(d - 2e-4)


def run_stream(ctx, cache, requests, max_views, max_inflight=2, budget=120 << 30,
               arena=2 << 30, hash_images=True):
    """Runs one request stream through a fresh server and returns its report.

    max_views == 1 is the plain per-request path (one request per launch,
    one launch at a time, each rendered by rt_render's kernel)."""
    wl = cache.wl
    cap = len(wl["pool"])
    srv = capi.Server(ctx, budget=budget, arena=arena, max_views=max_views,
                      max_inflight=max_inflight, max_scenes=cap)
    try:
        order, last, doomed = [], {}, set()
        clock = 0
        for spec in wl["pool"]:
            sid = srv.add_scene(cache.get(spec))
            clock += 1
            order.append(sid)
            last[sid] = clock
        srv.reset_stats()
        todo = queue.Queue()
        done, ups = {}, {}

        def collect():
            while True:
                item = todo.get()
                if item is None:
                    return
                k, tk, w, h = item
                img, info = srv.result(tk, w, h, raise_on_error=False)
                if w == 0:
                    ups[k] = (info.status, info.done_ms - info.submit_ms)
                    continue
                crc = zlib.crc32(img) if (hash_images and info.status == 0) else None
                done[k] = (info.status, info.submit_ms, info.start_ms, info.done_ms,
                           info.batch_views, info.rays, crc)

        th = threading.Thread(target=collect, daemon=True)
        th.start()
        t0 = time.perf_counter()
        for k, rq in enumerate(requests):
            _pace(t0, rq["t"])
            clock += 1
            if rq["kind"] == "render":
                cand = [s for s in order if s not in doomed]
                sid = cand[min(len(cand) - 1, int(rq["u"] * len(cand)))]
                last[sid] = clock
                tk = srv.submit_render(sid, rq["camera"], rq["width"], rq["height"],
                                       rq["max_bounces"])
                todo.put((k, tk, rq["width"], rq["height"]))
            else:
                live = [s for s in order if s not in doomed]
                while len(live) >= cap:
                    victim = min(live, key=last.get)
                    doomed.add(victim)
                    live.remove(victim)
                specs = wl["uploads"]
                tk, sid = srv.upload(cache.get(specs[rq["index"] % len(specs)]))
                order.append(sid)
                last[sid] = clock
                todo.put((k, tk, 0, 0))
        submit_s = time.perf_counter() - t0
        todo.put(None)
        th.join()
        st = srv.stats()
    finally:
        srv.close()
    rend = [v for v in done.values()]
    up_lat = [v[1] for v in ups.values() if v[0] == 0]
    up_fail = sum(v[0] != 0 for v in ups.values())
    ok = [v for v in rend if v[0] == 0]
    lat = np.array([v[3] - v[1] for v in ok]) if ok else np.zeros(1)
    span_ms = st.last_done_ms - st.first_submit_ms
    offered = requests[-1]["t"] if requests else 0.0
    return dict(
        requests=len(requests), renders=len(rend), uploads=len(requests) - len(rend),
        failed=len(rend) - len(ok), upload_failed=up_fail,
        p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)),
        mean_ms=float(lat.mean()), max_ms=float(lat.max()),
        server_p50_ms=st.p50_ms, server_p99_ms=st.p99_ms,
        upload_p50_ms=float(np.median(up_lat)) if up_lat else None,
        rays=int(st.rays), span_ms=span_ms, offered_s=offered, submit_s=submit_s,
        mrays_s=st.rays / (span_ms * 1e-3) / 1e6 if span_ms > 0 else 0.0,
        req_s=len(ok) / (span_ms * 1e-3) if span_ms > 0 else 0.0,
        launches=int(st.batches), mean_batch_views=st.mean_batch_views,
        evicted=int(st.evicted), resident_scenes=int(st.resident_scenes),
        crc={k: v[6] for k, v in done.items() if v[6] is not None})
