"""The spatial partition replay of the GPU builder, as a model (CPU only).

apply_spatial_split (src/builders/spatial_sah.rs:605-724) partitions a
task's references with a three-way swap loop, an equal-count fallback and a
straddler loop; the resulting order is part of the output. The GPU builder
does not move references while replaying those loops: it reads each
reference's class once and writes the final order directly (left references
in processing order, right ones from the back in processing order,
straddlers as a queue that every later left reference rotates by one). This
test checks that formulation against the literal loops on random class
sequences, split space, begins and both fallback forms."""
import random

L, R, M = 0, 1, 2
LEFT_FRAG, RIGHT_FRAG = 1 << 30, 2 << 30


def literal(cls, n, space, fix_fallback, begin):
    """The reference's loops on a permutation of slots (None: it panics)."""
    p = list(range(n)) + [0] * (space - n)
    i, le, rb, re = 0, 0, n, n
    while i < rb:
        e = p[i]
        if cls[e] == L:
            p[i], p[le] = p[le], e
            i += 1
            le += 1
        elif cls[e] == R:
            rb -= 1
            p[i], p[rb] = p[rb], e
        else:
            i += 1
    lc, rc = le, re - rb
    if (lc == 0 or rc == 0) and le == rb:
        if lc > 0:
            if fix_fallback:
                le = lc // 2
            elif lc // 2 < begin:
                return None
            else:
                le = lc // 2 - begin
        else:
            le += rc // 2
        rb = le
    while le < rb:
        e = p[le]
        if space - re > 0:
            p[re] = e | RIGHT_FRAG
            p[le] = e | LEFT_FRAG
            re += 1
            le += 1
            lc += 1
            rc += 1
        elif lc < rc:
            le += 1
            lc += 1
        else:
            rb -= 1
            p[le], p[rb] = p[rb], e
            rc += 1
    return p[:re], le, rb, re


def queue_form(cls, n, space, fix_fallback, begin):
    """sb_replay_ring in csrc/sbvh.cu."""
    out = [None] * space
    m = sum(1 for c in cls if c == M)
    queue, head = [], 0
    i = j = le = rc = 0
    while i + j < n:
        src, c, done = i, cls[i], False
        while c == R:
            out[n - 1 - rc] = src
            rc += 1
            j += 1
            if i + j >= n:
                done = True
                break
            src = n - j
            c = cls[src]
        if done:
            break
        if c == L:
            out[le] = src
            le += 1
            if len(queue) != head:
                queue.append(queue[head])
                head += 1
        else:
            queue.append(src)
        i += 1
    lc, rcnt = le, rc
    if (lc == 0 or rcnt == 0) and m == 0:
        if lc > 0:
            if fix_fallback:
                le = lc // 2
            elif lc // 2 < begin:
                return None
            else:
                le = lc // 2 - begin
        else:
            le += rcnt // 2
        return out[:n], le, le, n
    re, a, bp = n, 0, m
    cur = queue[head] if m else 0
    while a < bp:
        if space - re > 0:
            out[le + a] = cur | LEFT_FRAG
            out[re] = cur | RIGHT_FRAG
            re += 1
            a += 1
            lc += 1
            rcnt += 1
            if a < bp:
                cur = queue[head + a]
        elif lc < rcnt:
            out[le + a] = cur
            a += 1
            lc += 1
            if a < bp:
                cur = queue[head + a]
        else:
            bp -= 1
            out[le + bp] = cur
            rcnt += 1
            if a < bp:
                cur = queue[head + bp]
    return out[:re], le + a, le + bp, re


def test_queue_form_equals_the_literal_loops():
    rng = random.Random(1)
    panics = 0
    for _ in range(20000):
        n = rng.randint(1, 40)
        weights = [rng.random() for _ in range(3)]
        cls = rng.choices([L, R, M], weights=weights, k=n)
        space = n + rng.randint(0, 20)
        fix = rng.random() < 0.5
        begin = rng.randint(0, 5)
        want = literal(cls, n, space, fix, begin)
        assert queue_form(cls, n, space, fix, begin) == want, (cls, space, fix, begin)
        panics += want is None
    assert panics > 0  # the panicking fallback is among the cases
