"""Shared set-up for GPU tests of learned sizing: a sizing network trained on
a few synthetic batches of uneven scenes (labels from the exact count pass)."""


def train_sizer(sr, seeds, scenes_per_batch=24, epochs=40):
    xs, ts, keep = [], [], []
    for sd in seeds:
        b = sr.SceneBatch(mode=sr.MODE_PIXEL)
        b.add_synth(2, sd, scenes_per_batch)
        b.commit()
        xs.append(b.features())
        ts.append(b.labels())
        keep.append(b)
    x = sr.concat_device(xs)
    t = sr.concat_device(ts)
    sz = sr.Sizer(seed=11)
    sz.set_norm(sr.sizer_norm(x.numpy(), t.numpy()))
    losses = [sz.train(x, t, epochs=max(1, epochs // 4), batch=4096, seed=e) for e in range(4)]
    for b in keep:
        b.close()
    return sz, x, t, losses
