set output "hist_cfg1_MOTIF00012.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-73.8453:18.7222]
set yrange [0:163193]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00012.dat" using 1:2 title 'MOTIF00012 (cfg1)' with boxes
