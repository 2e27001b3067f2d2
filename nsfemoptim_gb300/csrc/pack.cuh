// A pack of steppers advanced by one graph launch: every stepper's time step is one branch of a
// single captured CUDA graph (fork and join through events during the capture), so independent
// flow instances -- on one mesh or on meshes of different resolution -- advance together with one
// cudaGraphLaunch per step.  The reference has no counterpart (its time loop drives one flow).
//
// Concurrent branches must not wait on one another: a solve on the whole-GPU cooperative grid
// spins on a software barrier that needs every SM, so a pack of more than one stepper only takes
// steppers whose solves stay inside thread-block clusters (NSF_PCG_PATH=auto-cluster at creation).
//
// Included at the end of capi.cu (it uses the stepper internals).
#pragma once

struct nsf_pack_s
{
    std::vector<nsf_chorin> S;
    std::vector<nsf_batch> Bt; // batches (nsf_pack_create_batches): one branch per batch
    cudaStream_t stream = nullptr;
    std::vector<cudaStream_t> branch;
    std::vector<cudaEvent_t> joined;
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernelsPerCapture = 0;

    ~nsf_pack_s()
    {
        if (exec)
            cudaGraphExecDestroy(exec);
        if (graph)
            cudaGraphDestroy(graph);
        for (cudaEvent_t e : joined)
            if (e)
                cudaEventDestroy(e);
        if (fork)
            cudaEventDestroy(fork);
        for (cudaStream_t b : branch)
            if (b)
                cudaStreamDestroy(b);
        if (stream)
            cudaStreamDestroy(stream);
    }

    void capture()
    {
        const long long before = launchCounter().load();
        NSF_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        try
        {
            NSF_CUDA(cudaEventRecord(fork, stream));
            const size_t n = S.size() + Bt.size();
            for (size_t i = 0; i < n; i++)
            {
                NSF_CUDA(cudaStreamWaitEvent(branch[i], fork, 0));
                if (i < S.size())
                    S[i]->enqueueStep(branch[i]);
                else
                    Bt[i - S.size()]->enqueueStep(branch[i]);
                NSF_CUDA(cudaEventRecord(joined[i], branch[i]));
                NSF_CUDA(cudaStreamWaitEvent(stream, joined[i], 0));
            }
        }
        catch (...)
        {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(stream, &g);
            if (g)
                cudaGraphDestroy(g);
            throw;
        }
        NSF_CUDA(cudaStreamEndCapture(stream, &graph));
        NSF_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        kernelsPerCapture = launchCounter().load() - before;
        launchCounter().fetch_sub(kernelsPerCapture); // counted when replayed
    }
};

extern "C" int nsf_pack_create(const nsf_chorin * steppers, int n, nsf_pack * out)
{
    return guarded([&] {
        require(steppers && out && n >= 1, "bad argument");
        auto p = std::make_unique<nsf_pack_s>();
        for (int i = 0; i < n; i++)
        {
            require(steppers[i] != nullptr, "null stepper in the pack");
            for (int j = 0; j < i; j++)
                require(steppers[j] != steppers[i], "a stepper appears twice in the pack");
            if (n > 1)
                require(!steppers[i]->usesGrid(),
                        "a packed stepper solves on the whole-GPU cooperative grid; create it with "
                        "NSF_PCG_PATH=auto-cluster so that its solves stay inside thread-block clusters");
            p->S.push_back(steppers[i]);
        }
        NSF_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
        NSF_CUDA(cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming));
        p->branch.resize(n, nullptr);
        p->joined.resize(n, nullptr);
        for (int i = 0; i < n; i++)
        {
            NSF_CUDA(cudaStreamCreateWithFlags(&p->branch[i], cudaStreamNonBlocking));
            NSF_CUDA(cudaEventCreateWithFlags(&p->joined[i], cudaEventDisableTiming));
        }
        p->capture();
        *out = p.release();
    });
}

extern "C" int nsf_pack_create_batches(const nsf_batch * batches, int n, nsf_pack * out)
{
    return guarded([&] {
        require(batches && out && n >= 1, "bad argument");
        auto p = std::make_unique<nsf_pack_s>();
        for (int i = 0; i < n; i++)
        {
            require(batches[i] != nullptr, "null batch in the pack");
            for (int j = 0; j < i; j++)
                require(batches[j] != batches[i], "a batch appears twice in the pack");
            p->Bt.push_back(batches[i]);
        }
        NSF_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
        NSF_CUDA(cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming));
        p->branch.resize(n, nullptr);
        p->joined.resize(n, nullptr);
        for (int i = 0; i < n; i++)
        {
            NSF_CUDA(cudaStreamCreateWithFlags(&p->branch[i], cudaStreamNonBlocking));
            NSF_CUDA(cudaEventCreateWithFlags(&p->joined[i], cudaEventDisableTiming));
        }
        p->capture();
        *out = p.release();
    });
}

extern "C" long long nsf_pack_kernels_per_step(nsf_pack p) { return p ? p->kernelsPerCapture : 0; }

extern "C" int nsf_pack_step(nsf_pack p, int nSteps, void * stream)
{
    return guarded([&] {
        require(p && nSteps >= 0, "bad argument");
        cudaStream_t s = stream ? asStream(stream) : p->stream;
        for (int i = 0; i < nSteps; i++)
        {
            NSF_CUDA(cudaGraphLaunch(p->exec, s));
            launchCounter().fetch_add(p->kernelsPerCapture, std::memory_order_relaxed);
        }
    });
}

extern "C" void nsf_pack_destroy(nsf_pack p) { delete p; }
