"""Client side of the served form: drives an rt_server with a timed request
stream (``scenes.served_requests``) and collects results on a second thread.

The client keeps a mirror of the server's recency order (every add_scene and
submit advances it by one, as the server's submission clock does) so that it
never targets a scene that an upload has displaced under the scene cap, and
an uploaded scene becomes a render target a fixed number of requests after
its upload, waiting for the upload if needed.  The sequence of scenes,
cameras, sizes and depths is therefore the same for every server
configuration, and images can be compared request by request."""
import collections
import queue
import threading
import time
import zlib

import numpy as np

from . import capi

UPLOAD_LAG = 10   # requests between an upload and its first render


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
        done = {}

        def collect():
            while True:
                item = todo.get()
                if item is None:
                    return
                k, tk, w, h = item
                img, info = srv.result(tk, w, h, raise_on_error=False)
                crc = zlib.crc32(img) if (hash_images and info.status == 0) else None
                done[k] = (info.status, info.submit_ms, info.start_ms, info.done_ms,
                           info.batch_views, info.rays, crc)

        th = threading.Thread(target=collect, daemon=True)
        th.start()
        uploads = collections.deque()       # (first target index, ticket, key)
        up_lat, up_fail = [], 0
        t0 = time.perf_counter()
        for k, rq in enumerate(requests):
            while uploads and uploads[0][0] <= k:
                _, tk, key = uploads.popleft()
                _, info = srv.result(tk, raise_on_error=False)
                i = order.index(key)
                if info.status == 0:
                    up_lat.append(info.done_ms - info.submit_ms)
                    order[i] = info.scene_id
                    last[info.scene_id] = last.pop(key)
                    if key in doomed:
                        doomed.discard(key)
                        doomed.add(info.scene_id)
                else:
                    up_fail += 1
                    order.pop(i)
                    last.pop(key)
                    doomed.discard(key)
            _pace(t0, rq["t"])
            clock += 1
            if rq["kind"] == "render":
                cand = [s for s in order if isinstance(s, int) and s not in doomed]
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
                ups = wl["uploads"]
                tk = srv.submit_upload(cache.get(ups[rq["index"] % len(ups)]))
                key = ("upload", tk)
                order.append(key)
                last[key] = clock
                uploads.append((k + UPLOAD_LAG, tk, key))
        for _, tk, _ in uploads:
            _, info = srv.result(tk, raise_on_error=False)
            if info.status == 0:
                up_lat.append(info.done_ms - info.submit_ms)
            else:
                up_fail += 1
        todo.put(None)
        th.join()
        st = srv.stats()
    finally:
        srv.close()
    rend = [v for v in done.values()]
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
        rays=int(st.rays), span_ms=span_ms, offered_s=offered,
        mrays_s=st.rays / (span_ms * 1e-3) / 1e6 if span_ms > 0 else 0.0,
        req_s=len(ok) / (span_ms * 1e-3) if span_ms > 0 else 0.0,
        launches=int(st.batches), mean_batch_views=st.mean_batch_views,
        evicted=int(st.evicted), resident_scenes=int(st.resident_scenes),
        crc={k: v[6] for k, v in done.items() if v[6] is not None})
