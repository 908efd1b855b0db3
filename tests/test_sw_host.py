"""Host logic of the shallow-water drop-in (no GPU)."""


def test_sw_cotangent_sum_to_broadcast_shape():
    """SW.step_adj returns the H / h_wind cotangents summed down to the shapes
    the inputs were given in (jax.vjp of a broadcast input)."""
    import torch
    from vardyn_gb300.model_qgsw.sw import SW
    a = torch.arange(2 * 3 * 4, dtype=torch.float64).reshape(2, 3, 4)
    assert torch.equal(SW._sum_to(a, (2, 3, 4)), a)
    assert torch.equal(SW._sum_to(a, (1, 3, 4)), a.sum(0, keepdim=True))
    assert torch.equal(SW._sum_to(a, (3, 4)), a.sum(0))
    assert torch.equal(SW._sum_to(a, (2, 1, 1)), a.sum((1, 2), keepdim=True))
    assert torch.equal(SW._sum_to(a, (2, 1, 4)), a.sum(1, keepdim=True))
