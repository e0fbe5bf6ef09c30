"""Learned proposal (gvr.proposal): a short training run on renders from
this rasteriser must lower the network's loss, and on held-out parameter
draws the trained proposal must start the fit closer to the ground truth
than the mean does (lower photometric RMSE at step 0, lower parameter
error) -- what the network gains over the fit without it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_proposal_trains_and_beats_the_mean_start():
    import torch
    from gvr import fitting, proposal, tc
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    model = fitting.MorphableModel(num_vertices=2562, seed=0, device=dev)
    net = proposal.ProposalNet(dev, seed=0)
    trainer = proposal.Trainer(model, net, batch=64, lr=1e-3, seed=1)
    losses, secs = trainer.train(300, log_every=50)
    assert tc.tc_error() == 0
    first, last = losses[0][1], losses[-1][1]
    assert last < 0.95 * first, losses

    fitter = fitting.Fitter(model, num_views=4, size=128)
    seeds = list(range(10_000, 10_016))
    gt = np.concatenate([fitting.sample_params(np.random.default_rng(s), 1) for s in seeds])
    p = torch.from_numpy(gt).to(dev)
    with torch.no_grad():
        target = fitter.render(p)
        pred = net.predict(proposal.mosaic(trainer.view_fitter.render(p)))
        mean = torch.from_numpy(fitting.mean_params(len(seeds))).to(dev)
        rm_pred = torch.sqrt(fitter.loss(fitter.render(pred), target))
        rm_mean = torch.sqrt(fitter.loss(fitter.render(mean), target))
    sd = net.sd.clamp_min(1e-6)
    active = net.sd > 0
    err_pred = (((pred - p) / sd)[:, active] ** 2).mean()
    err_mean = (((mean - p) / sd)[:, active] ** 2).mean()
    assert float(err_pred) < float(err_mean)
    assert float(rm_pred.mean()) < float(rm_mean.mean())


def test_trainer_checkpoint_resume(tmp_path):
    """A checkpoint restores the weights, the Adam state, the sampler's RNG
    and the step count: the resumed trainer draws the same next batch and
    holds the same optimiser state as the one that wrote it."""
    import torch
    from gvr import fitting, proposal
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    model = fitting.MorphableModel(num_vertices=2562, seed=0, device=dev)
    a = proposal.Trainer(model, proposal.ProposalNet(dev, seed=0), batch=16, lr=1e-3, seed=3)
    a.train(40)
    path = tmp_path / "proposal.pt"
    a.checkpoint(path)
    b = proposal.Trainer(model, proposal.ProposalNet(dev, seed=5), batch=16, lr=2e-3, seed=9)
    b.resume(path)
    assert b.steps_done == a.steps_done == 40
    for x, y in zip(a.net.parameters(), b.net.parameters()):
        assert torch.equal(x.detach(), y.detach())
    sa, sb = a.opt.state_dict(), b.opt.state_dict()
    for k in sa["state"]:
        for name in ("exp_avg", "exp_avg_sq"):
            assert torch.equal(sa["state"][k][name].cpu(), sb["state"][k][name].cpu())
    pa, _ = a.sample(4)
    pb, _ = b.sample(4)
    assert torch.equal(pa, pb)
    losses, _ = b.train(50, start=b.steps_done)
    assert b.steps_done == 50
