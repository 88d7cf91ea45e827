"""Parameter-server protocol of the reference (3rdparty/protobuf/args.proto,
src/streamWorker.cpp): protobuf wire codec, SP request/reply over TCP, the
worker loop (streamWorker/gpuWorker) and a parameter server."""
