#define GIT_COMMIT_HASH "oracle"
#define GIT_BRANCH "oracle"
